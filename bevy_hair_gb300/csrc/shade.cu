// Shade pass: per-pixel Karis-fit Marschner R/TT/TRT with Zinke dual
// scattering and the deep-opacity optical depth toward the key light
// (shade.wesl:31-593).  Output colour is compared with a tolerance, so this
// file compiles with FMA contraction on.
#include <cuda_runtime.h>

#include <cstring>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "hg_device.cuh"
#include "hg_internal.h"
#include "hg_mlp.cuh"
#include "hg_mlp_small.cuh"
#include "hg_mlp_tc.cuh"

namespace hg {
namespace {

constexpr float kIor = 1.55f;
constexpr float kDensityFront = 0.7f;
constexpr float kDensityBack = 0.7f;
constexpr int kScatterSteps = 8;

struct Lobes {
    f3 r, tt, trt;
};
struct Shape {
    f3 alpha, beta;
};
struct Dual {
    Lobes fwd;
    f3 a_f, beta_f2, a_back, delta_b, sigma_b2;
};

__device__ __forceinline__ f3 spl(float s) { return {s, s, s}; }
__device__ __forceinline__ f3 vmul(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 vdiv(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ f3 vexp(f3 a) { return {expf(a.x), expf(a.y), expf(a.z)}; }
__device__ __forceinline__ f3 vsqrt(f3 a) { return {sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)}; }
__device__ __forceinline__ f3 vmaxs(f3 a, float s) { return {fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)}; }
__device__ __forceinline__ f3 vmins(f3 a, float s) { return {fminf(a.x, s), fminf(a.y, s), fminf(a.z, s)}; }
__device__ __forceinline__ f3 ld3(const float* v) { return {v[0], v[1], v[2]}; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// gaussian3 (shade.wesl:51-54)
__device__ __forceinline__ f3 gaussian3(f3 b, f3 x) {
    f3 bb = vmaxs(b, 1e-3f);
    const float k = 2.50662827f;  // sqrt(2 pi)
    f3 num = vexp(vdiv(vmul(mul3s(x, -0.5f), x), vmul(bb, bb)));
    return vdiv(num, mul3s(bb, k));
}

// fresnel (shade.wesl:56-60), the fifth power by multiplication.
__device__ __forceinline__ float fresnel(float cos_t) {
    const float r0 = (1.0f - kIor) / (1.0f + kIor);
    const float f0 = r0 * r0;
    float m = 1.0f - clampf(cos_t, 0.0f, 1.0f);
    float m2 = m * m;
    return f0 + (1.0f - f0) * (m2 * m2 * m);
}

// absorption_from_color (shade.wesl:70-77)
__device__ __forceinline__ f3 absorption_from_color(f3 c, float roughness) {
    float b = clampf(roughness, 0.0f, 1.0f);
    float b2 = b * b;
    float b3 = b2 * b;
    float d = 5.969f - 0.215f * b + 2.532f * b2 - 10.73f * b3 + 5.574f * b2 * b2 + 0.245f * b3 * b2;
    f3 l = {logf(clampf(c.x, 1e-4f, 1.0f)) / d, logf(clampf(c.y, 1e-4f, 1.0f)) / d,
            logf(clampf(c.z, 1e-4f, 1.0f)) / d};
    return vmul(l, l);
}

// azimuthal (shade.wesl:94-116)
__device__ __forceinline__ Lobes azimuthal(float cos_theta_d, float cos_phi, f3 sigma_a) {
    float cos_half_phi = sqrtf(clampf(0.5f + 0.5f * cos_phi, 0.0f, 1.0f));
    float n_r = 0.25f * cos_half_phi * fresnel(cos_theta_d * cos_half_phi);
    float inv_ctd = 1.0f / cos_theta_d;
    float eta = 1.19f * inv_ctd + 0.36f * cos_theta_d;
    float a = 1.0f / eta;
    float h = cos_half_phi * (1.0f + a * (0.6f - 0.8f * cos_phi));
    float f_tt = fresnel(cos_theta_d * sqrtf(clampf(1.0f - h * h, 0.0f, 1.0f)));
    float path = 2.0f * sqrtf(clampf(1.0f - h * h * a * a, 0.0f, 1.0f)) * inv_ctd;
    float k_tt = expf(-3.65f * cos_phi - 3.98f) * (1.0f - f_tt) * (1.0f - f_tt);
    float f_trt = fresnel(cos_theta_d * 0.5f);
    float k_trt = expf(17.0f * cos_phi - 16.78f) * (1.0f - f_trt) * (1.0f - f_trt) * f_trt;
    float trt_path = 3.2f * inv_ctd;
    Lobes r;
    r.r = spl(n_r);
    r.tt = {expf(-sigma_a.x * path) * k_tt, expf(-sigma_a.y * path) * k_tt, expf(-sigma_a.z * path) * k_tt};
    r.trt = {expf(-sigma_a.x * trt_path) * k_trt, expf(-sigma_a.y * trt_path) * k_trt,
             expf(-sigma_a.z * trt_path) * k_trt};
    return r;
}

__device__ __forceinline__ Shape lobe_shape(float roughness, float tilt) {
    float b = clampf(roughness * roughness, 0.02f, 1.0f);
    return {{tilt, -0.5f * tilt, -1.5f * tilt}, {b, 0.5f * b, 2.0f * b}};
}

__device__ __forceinline__ f3 lobe_mean(const Lobes& l, f3 total, f3 q) {
    f3 num = add3(add3(mul3s(l.r, q.x), mul3s(l.tt, q.y)), mul3s(l.trt, q.z));
    return vdiv(num, vmaxs(total, 1e-5f));
}

// The azimuthal angles dual_scatter integrates over are fixed: per step i,
// cos phi at u = (i + 0.5) / kScatterSteps for the back half (phi = u pi/2)
// and the front half (phi = (1 + u) pi/2), with the factors of azimuthal()
// that depend on phi alone: cos(phi/2), exp(-3.65 cos phi - 3.98) and
// exp(17 cos phi - 16.78).  Filled from double precision on the host.
struct ScatterAngle {
    float cos_phi, cos_half_phi, k_tt, k_trt;
};
__constant__ ScatterAngle c_scatter[2 * kScatterSteps];  // [0, steps): back, [steps, 2 steps): front

// azimuthal() at one of those angles, with the terms that depend only on the
// pixel (cos theta_d, sigma_a) computed once by the caller.
struct AzimuthPixel {
    float cos_theta_d, inv_ctd, a;
    f3 sigma_a;
    f3 trt;  // exp(-sigma_a 3.2 / cos theta_d) (1 - F)^2 F with F = fresnel(cos theta_d / 2)
};

__device__ __forceinline__ AzimuthPixel azimuth_pixel(float cos_theta_d, f3 sigma_a) {
    AzimuthPixel q;
    q.cos_theta_d = cos_theta_d;
    q.inv_ctd = 1.0f / cos_theta_d;
    const float eta = 1.19f * q.inv_ctd + 0.36f * cos_theta_d;
    q.a = 1.0f / eta;
    q.sigma_a = sigma_a;
    const float f_trt = fresnel(cos_theta_d * 0.5f);
    const float trt_path = 3.2f * q.inv_ctd;
    const float k = (1.0f - f_trt) * (1.0f - f_trt) * f_trt;
    q.trt = {expf(-sigma_a.x * trt_path) * k, expf(-sigma_a.y * trt_path) * k, expf(-sigma_a.z * trt_path) * k};
    return q;
}

__device__ __forceinline__ Lobes azimuthal_at(const AzimuthPixel& q, const ScatterAngle& g) {
    const float n_r = 0.25f * g.cos_half_phi * fresnel(q.cos_theta_d * g.cos_half_phi);
    const float h = g.cos_half_phi * (1.0f + q.a * (0.6f - 0.8f * g.cos_phi));
    const float f_tt = fresnel(q.cos_theta_d * sqrtf(clampf(1.0f - h * h, 0.0f, 1.0f)));
    const float path = 2.0f * sqrtf(clampf(1.0f - h * h * q.a * q.a, 0.0f, 1.0f)) * q.inv_ctd;
    const float k_tt = g.k_tt * (1.0f - f_tt) * (1.0f - f_tt);
    Lobes r;
    r.r = spl(n_r);
    r.tt = {expf(-q.sigma_a.x * path) * k_tt, expf(-q.sigma_a.y * path) * k_tt, expf(-q.sigma_a.z * path) * k_tt};
    r.trt = mul3s(q.trt, g.k_trt);
    return r;
}

// dual_scatter (shade.wesl:153-190)
__device__ Dual dual_scatter(float cos_theta_d, f3 sigma_a, const Shape& shape) {
    Lobes fwd = {spl(0.0f), spl(0.0f), spl(0.0f)}, back = fwd;
    const AzimuthPixel q = azimuth_pixel(cos_theta_d, sigma_a);
#pragma unroll 2
    for (int i = 0; i < kScatterSteps; ++i) {
        Lobes b = azimuthal_at(q, c_scatter[i]);
        Lobes f = azimuthal_at(q, c_scatter[kScatterSteps + i]);
        back.r = add3(back.r, b.r);
        back.tt = add3(back.tt, b.tt);
        back.trt = add3(back.trt, b.trt);
        fwd.r = add3(fwd.r, f.r);
        fwd.tt = add3(fwd.tt, f.tt);
        fwd.trt = add3(fwd.trt, f.trt);
    }
    const float w = kPi / (float)kScatterSteps;
    fwd = {mul3s(fwd.r, w), mul3s(fwd.tt, w), mul3s(fwd.trt, w)};
    back = {mul3s(back.r, w), mul3s(back.tt, w), mul3s(back.trt, w)};
    Dual d;
    d.fwd = fwd;
    f3 a_f = vmins(add3(add3(fwd.r, fwd.tt), fwd.trt), 0.95f);
    f3 a_b = add3(add3(back.r, back.tt), back.trt);
    f3 beta2 = vmul(shape.beta, shape.beta);
    f3 beta_f2 = lobe_mean(fwd, a_f, beta2);
    f3 alpha_b = lobe_mean(back, a_b, shape.alpha);
    f3 beta_b2 = lobe_mean(back, a_b, beta2);
    f3 af2 = vmul(a_f, a_f);
    f3 rest = {1.0f - af2.x, 1.0f - af2.y, 1.0f - af2.z};
    f3 ab2 = vmul(a_b, a_b);
    f3 ab3 = vmul(ab2, a_b);
    f3 rr = vmul(rest, rest);
    f3 rest3 = vmul(rr, rest);
    f3 a_back = add3(vdiv(vmul(a_b, af2), rest), vdiv(vmul(ab3, af2), rest3));
    f3 t1 = {1.0f - 2.0f * ab2.x / rr.x, 1.0f - 2.0f * ab2.y / rr.y, 1.0f - 2.0f * ab2.z / rr.z};
    f3 num2 = add3(mul3s(rr, 2.0f), vmul(mul3s(af2, 4.0f), ab2));
    f3 delta_b = add3(vmul(alpha_b, t1), vdiv(vmul(alpha_b, num2), rest3));
    f3 beta_f = vsqrt(beta_f2), beta_b = vsqrt(beta_b2);
    f3 lead = add3(spl(1.0f), mul3s(af2, kDensityBack));
    f3 s1 = vsqrt(add3(mul3s(beta_f2, 2.0f), beta_b2));
    f3 s2 = vsqrt(add3(mul3s(beta_f2, 2.0f), mul3s(beta_b2, 3.0f)));
    f3 numer = vmul(lead, add3(vmul(a_b, s1), vmul(ab3, s2)));
    f3 den = vmaxs(add3(a_b, vmul(ab3, add3(mul3s(beta_f, 2.0f), mul3s(beta_b, 3.0f)))), 1e-5f);
    f3 sigma_b = vdiv(numer, den);
    d.a_f = a_f;
    d.beta_f2 = beta_f2;
    d.a_back = a_back;
    d.delta_b = delta_b;
    d.sigma_b2 = vmul(sigma_b, sigma_b);
    return d;
}

// Angles of one light at a fibre (shade.wesl:196-206).
struct Geometry {
    float sin_i, sin_o, theta_h, cos_theta_d, cos_phi;
};

// t and v arrive normalized (once per pixel); the light direction per light.
__device__ __forceinline__ Geometry light_geometry(f3 t, f3 v, f3 light) {
    f3 l = safe_normalize(light);
    Geometry g;
    g.sin_i = clampf(dot3(t, l), -1.0f, 1.0f);
    g.sin_o = clampf(dot3(t, v), -1.0f, 1.0f);
    float theta_i = asinf(g.sin_i);
    float theta_o = asinf(g.sin_o);
    g.theta_h = theta_i + theta_o;
    g.cos_theta_d = fmaxf(cosf(0.5f * fabsf(theta_i - theta_o)), 1e-3f);
    f3 t_i = sub3(l, mul3s(t, g.sin_i));
    f3 t_o = sub3(v, mul3s(t, g.sin_o));
    float proj = sqrtf(fmaxf(dot3(t_i, t_i) * dot3(t_o, t_o), 1e-8f));
    g.cos_phi = clampf(dot3(t_i, t_o) / proj, -1.0f, 1.0f);
    return g;
}

// Forward-scattered spread through `depth` of hair in front of the fibre
// (shade.wesl:228-242).
__device__ f3 spread_term(const Shape& shape, const Dual& ds, float theta_h, float depth, float direct) {
    f3 x = spl(theta_h);
    f3 sigma_f2 = mul3s(ds.beta_f2, depth);
    f3 transmit = {powf(ds.a_f.x, depth), powf(ds.a_f.y, depth), powf(ds.a_f.z, depth)};
    f3 beta2 = vmul(shape.beta, shape.beta);
    f3 g0 = gaussian3(vsqrt(add3(spl(beta2.x), sigma_f2)), sub3(x, spl(shape.alpha.x)));
    f3 g1 = gaussian3(vsqrt(add3(spl(beta2.y), sigma_f2)), sub3(x, spl(shape.alpha.y)));
    f3 g2 = gaussian3(vsqrt(add3(spl(beta2.z), sigma_f2)), sub3(x, spl(shape.alpha.z)));
    f3 spread = add3(add3(vmul(g0, ds.fwd.r), vmul(g1, ds.fwd.tt)), vmul(g2, ds.fwd.trt));
    f3 gb = gaussian3(vsqrt(add3(ds.sigma_b2, sigma_f2)), sub3(x, ds.delta_b));
    f3 back_spread = mul3s(vmul(ds.a_back, gb), 2.0f / kPi);
    f3 inner = add3(mul3s(spread, 1.0f / kPi), mul3s(back_spread, kPi * kDensityBack));
    return vmul(mul3s(transmit, (1.0f - direct) * kDensityFront), inner);
}

// hair_bsdf (shade.wesl:193-244); t_n and v_n are the normalized tangent and view.
__device__ __forceinline__ f3 hair_bsdf(f3 t_n, f3 v_n, f3 light, f3 sigma_a, const Shape& shape, const Dual& ds,
                                        float depth) {
    const Geometry gm = light_geometry(t_n, v_n, light);
    Lobes n = azimuthal(gm.cos_theta_d, gm.cos_phi, sigma_a);
    f3 x = spl(gm.theta_h);
    f3 m = gaussian3(shape.beta, sub3(x, shape.alpha));
    f3 single = add3(add3(mul3s(n.r, m.x), mul3s(n.tt, m.y)), mul3s(n.trt, m.z));
    f3 g = gaussian3(vsqrt(ds.sigma_b2), sub3(x, ds.delta_b));
    f3 back = mul3s(vmul(ds.a_back, g), 2.0f / kPi);
    float direct = expf(-depth);
    f3 color = mul3s(add3(single, mul3s(back, kDensityBack)), direct);
    if (depth > 1e-3f) color = add3(color, spread_term(shape, ds, gm.theta_h, depth, direct));
    return color;
}

// ---------------------------------------------------------------- light probe
// probe_radiance (shade.wesl:330-427, the ENVIRONMENT_MAP specialization)
// over RGB9E5 cubemaps: major-axis face selection, bilinear within the face
// with clamp-to-edge, linear between mip levels.

struct EnvArgs {
    const uint32_t* spec;
    const uint32_t* diff;
    uint32_t spec_size, spec_levels, diff_size, diff_levels;
    float rot[4];
    float intensity;
};

__device__ __forceinline__ f3 rgb9e5(uint32_t w) {
    const int e = (int)(w >> 27) - 24;
    return {ldexpf((float)(w & 0x1ffu), e), ldexpf((float)((w >> 9) & 0x1ffu), e),
            ldexpf((float)((w >> 18) & 0x1ffu), e)};
}

// Direction -> face (+X -X +Y -Y +Z -Z) and (s, t) in [0, 1].
__device__ __forceinline__ int cube_face_uv(f3 d, float& s, float& t) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int face;
    float ma, sc, tc;
    if (ax >= ay && ax >= az) {
        face = d.x >= 0.0f ? 0 : 1;
        ma = ax;
        sc = d.x >= 0.0f ? -d.z : d.z;
        tc = -d.y;
    } else if (ay >= az) {
        face = d.y >= 0.0f ? 2 : 3;
        ma = ay;
        sc = d.x;
        tc = d.y >= 0.0f ? d.z : -d.z;
    } else {
        face = d.z >= 0.0f ? 4 : 5;
        ma = az;
        sc = d.z >= 0.0f ? d.x : -d.x;
        tc = -d.y;
    }
    const float inv = 1.0f / fmaxf(ma, 1e-20f);
    s = 0.5f * (sc * inv + 1.0f);
    t = 0.5f * (tc * inv + 1.0f);
    return face;
}

__device__ __forceinline__ f3 cube_bilinear(const uint32_t* __restrict__ level, uint32_t n, int face, float s,
                                            float t) {
    const float u = s * (float)n - 0.5f, v = t * (float)n - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float wu = u - fu, wv = v - fv;
    const int last = (int)n - 1;
    const int x0 = min(max((int)fu, 0), last), x1 = min(max((int)fu + 1, 0), last);
    const int y0 = min(max((int)fv, 0), last), y1 = min(max((int)fv + 1, 0), last);
    const uint32_t* f = level + (size_t)face * n * n;
    const f3 c00 = rgb9e5(__ldg(f + y0 * n + x0)), c10 = rgb9e5(__ldg(f + y0 * n + x1));
    const f3 c01 = rgb9e5(__ldg(f + y1 * n + x0)), c11 = rgb9e5(__ldg(f + y1 * n + x1));
    const f3 a = add3(mul3s(c00, 1.0f - wu), mul3s(c10, wu));
    const f3 b = add3(mul3s(c01, 1.0f - wu), mul3s(c11, wu));
    return add3(mul3s(a, 1.0f - wv), mul3s(b, wv));
}

__device__ f3 sample_cube(const uint32_t* __restrict__ texels, uint32_t size, uint32_t levels, f3 dir, float lod) {
    float s, t;
    const int face = cube_face_uv(dir, s, t);
    lod = clampf(lod, 0.0f, (float)(levels - 1));
    const uint32_t l0 = (uint32_t)lod, l1 = min(l0 + 1u, levels - 1u);
    const float w = lod - (float)l0;
    size_t off = 0;
    for (uint32_t l = 0; l < l0; ++l) {
        const size_t n = max(size >> l, 1u);
        off += 6 * n * n;
    }
    const uint32_t n0 = max(size >> l0, 1u);
    const f3 a = cube_bilinear(texels + off, n0, face, s, t);
    if (l1 == l0 || w <= 0.0f) return a;
    off += 6 * (size_t)n0 * n0;
    const f3 b = cube_bilinear(texels + off, max(size >> l1, 1u), face, s, t);
    return add3(mul3s(a, 1.0f - w), mul3s(b, w));
}

// quat_rotate + the left-handed flip (shade.wesl:329-339)
__device__ __forceinline__ f3 cubemap_dir(const float q[4], f3 dir) {
    const f3 qv = {q[0], q[1], q[2]};
    const f3 t = mul3s(cross3(qv, dir), 2.0f);
    f3 r = add3(add3(dir, mul3s(t, q[3])), cross3(qv, t));
    r.z = -r.z;
    return r;
}

// scatter_tint (shade.wesl:81-85) with luminance (:62-64)
__device__ __forceinline__ f3 scatter_tint(f3 albedo, float shadow) {
    const float lum = albedo.x * 0.2126f + albedo.y * 0.7152f + albedo.z * 0.0722f;
    const f3 hue = mul3s(albedo, 1.0f / fmaxf(lum, 1e-4f));
    const float e = 0.5f - 0.5f * clampf(shadow, 0.0f, 1.0f);
    return {powf(hue.x, e), powf(hue.y, e), powf(hue.z, e)};
}

__device__ f3 probe_radiance(const EnvArgs& env, f3 tangent, f3 fiber_n, f3 view, f3 albedo, float roughness,
                             float tilt) {
    const float theta_o = asinf(clampf(dot3(tangent, view), -1.0f, 1.0f));
    const float theta_i = tilt - theta_o;
    const f3 spec_dir = cubemap_dir(env.rot, add3(mul3s(tangent, sinf(theta_i)), mul3s(fiber_n, cosf(theta_i))));
    const f3 diff_dir = cubemap_dir(env.rot, fiber_n);
    const f3 spec = sample_cube(env.spec, env.spec_size, env.spec_levels, spec_dir,
                                roughness * (float)(env.spec_levels - 1));
    const f3 diff = sample_cube(env.diff, env.diff_size, env.diff_levels, diff_dir, 0.0f);
    const float cos_o = fmaxf(cosf(theta_o), 1e-3f);
    const float f_r = fresnel(cos_o);
    const float f_trt = fresnel(cos_o * 0.5f);
    const f3 sigma_a = absorption_from_color(albedo, roughness);
    const float k = 0.76f * (1.0f - f_trt) * (1.0f - f_trt) * f_trt;
    const f3 trt = {k * expf(-sigma_a.x * 3.2f / cos_o), k * expf(-sigma_a.y * 3.2f / cos_o),
                    k * expf(-sigma_a.z * 3.2f / cos_o)};
    const f3 scatter = vmul(albedo, scatter_tint(albedo, 0.5f));
    const f3 r = add3(vmul(spec, add3(spl(f_r), trt)), vmul(diff, scatter));
    return mul3s(r, env.intensity);
}

__device__ __forceinline__ float pixel_ao(const hg_hair_params& p, uint32_t low) {
    return p.flags[2] == 0u ? 1.0f : (float)(low & 0x3fu) / 63.0f;
}

// dom_texel_visibility (shade.wesl:262-277)
__device__ __forceinline__ float dom_texel_visibility(const uint32_t* __restrict__ dom, float sigma, int32_t x,
                                                      int32_t y, float dist, float near_, float far_,
                                                      uint32_t dom_w, uint32_t dom_h) {
    if (x < 0 || y < 0 || x >= (int32_t)dom_w || y >= (int32_t)dom_h) return 1.0f;
    uint32_t pix = (uint32_t)y * dom_w + (uint32_t)x;
    uint32_t front_q = __ldg(&dom[pix]);
    if (front_q == kDomEmpty) return 1.0f;
    float z_front = dequantize_depth(front_q, near_, far_);
    float thickness = fmaxf(far_ - near_, 1e-3f) / (float)kDomLayers;
    float rel = fmaxf((dist - z_front) - thickness * 0.05f, 0.0f);
    float t = rel / thickness;
    // Counters start at word dom_w*dom_h, which need not be 16-byte aligned.
    const uint32_t* c = dom + (size_t)dom_w * dom_h + (size_t)pix * kDomLayers;
    float occ = 0.0f;
#pragma unroll
    for (int k = 0; k < (int)kDomLayers; ++k) {
        float i = (float)k;
        if (!(i < t)) break;
        float count = __uint2float_rn(__ldg(c + k));
        occ += i + 1.0f <= t ? count : count * (t - i);
    }
    return expf(-occ * sigma);
}

// dom_visibility (shade.wesl:279-310)
__device__ float dom_visibility(const hg_hair_params& p, const uint32_t* __restrict__ dom, f3 world, float beta) {
    if (p.flags[3] == 0u) return 1.0f;
    float4 clip = mat_mul(p.light_clip_from_world, world.x, world.y, world.z, 1.0f);
    if (clip.w <= 0.0f) return 1.0f;
    float nx = clip.x / clip.w, ny = clip.y / clip.w;
    float ux = nx * 0.5f + 0.5f, uy = 1.0f - (ny * 0.5f + 0.5f);
    if (ux < 0.0f || uy < 0.0f || ux > 1.0f || uy > 1.0f) return 1.0f;
    uint32_t dom_w = f2u(p.dom_info[0]), dom_h = f2u(p.dom_info[1]);
    float near_ = p.dom_info[2], far_ = p.dom_info[3];
    float dist = dot3(sub3(world, ld3(p.light_eye)), ld3(p.light_forward)) -
                 (-logf(fmaxf(beta, 1e-4f)) * p.filter_params[2]);
    float fx = ux * (float)dom_w - 0.5f, fy = uy * (float)dom_h - 0.5f;
    float flx = floorf(fx), fly = floorf(fy);
    int32_t x0 = f2i(flx), y0 = f2i(fly);
    float tx = fx - flx, ty = fy - fly;
    float sigma = p.filter_params[3];
    float v00 = dom_texel_visibility(dom, sigma, x0, y0, dist, near_, far_, dom_w, dom_h);
    float v10 = dom_texel_visibility(dom, sigma, x0 + 1, y0, dist, near_, far_, dom_w, dom_h);
    float v01 = dom_texel_visibility(dom, sigma, x0, y0 + 1, dist, near_, far_, dom_w, dom_h);
    float v11 = dom_texel_visibility(dom, sigma, x0 + 1, y0 + 1, dist, near_, far_, dom_w, dom_h);
    return mixf(mixf(v00, v10, tx), mixf(v01, v11, tx), ty);
}

// Smooth range window and inverse-square falloff (Karis 2013; Lagarde and
// de Rousiers 2014), standing in for bevy_pbr's getDistanceAttenuation.
__device__ __forceinline__ float range_window(float dist2, float inv_range2) {
    float factor = dist2 * inv_range2;
    float s = clampf(1.0f - factor * factor, 0.0f, 1.0f);
    return s * s;
}

struct ShadeArgs {
    hg_hair_params p;
    const unsigned long long* center;
    const uint32_t* beta;
    const uint32_t* dom;
    const hg_light* lights;
    float4* shaded;
    float* shaded_depth;
    uint32_t n_lights;
    uint32_t ortho;
    float exposure;
};

// fs (shade.wesl:523-593) for pixel (x, y) of view v (fields p, center,
// beta, dom, shaded, shaded_depth).  Lights arrive sorted by kind (point,
// spot, directional, rect), the order the reference's loops visit them.
template <class V>
__device__ __forceinline__ void shade_pixel(const V& a, const hg_light* __restrict__ lights, uint32_t n_lights,
                                            uint32_t ortho, float exposure, const EnvArgs& env, uint32_t x,
                                            uint32_t y) {
    const hg_hair_params& p = a.p;
    const uint32_t width = f2u(p.screen[0]), height = f2u(p.screen[1]);
    if (x >= width || y >= height) return;
    const uint32_t pix = y * width + x;
    const unsigned long long word = __ldg(&a.center[pix]);
    if (is_empty(word)) {
        a.shaded[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a.shaded_depth[pix] = 0.0f;
        return;
    }
    const uint32_t low = (uint32_t)word, high = (uint32_t)(word >> 32);
    const uint32_t depth_q = high >> 8u;
    const float view_dist = dequantize_depth(depth_q, p.screen[2], p.screen[3]);
    const f3 world = reconstruct_world(p, (int32_t)x, (int32_t)y, view_dist);
    const f3 tangent = oct_decode(high & 0xffu, low >> 24u);
    const float uvw_z = (float)((low >> 6u) & 0x3fu) / 63.0f;
    const float beta = (float)(__ldg(&a.beta[pix]) & 0xffu) / 255.0f;
    const float roughness = fmaxf(p.appearance[0] * (0.65f + 0.7f * uvw_z), 0.04f);
    const float tilt = p.appearance[1];
    const float ascale = 0.65f + 0.35f * uvw_z;
    const f3 albedo = {p.albedo[0] * ascale, p.albedo[1] * ascale, p.albedo[2] * ascale};
    f3 view;
    if (ortho) {
        view = safe_normalize(mk3(p.clip_from_world[2], p.clip_from_world[6], p.clip_from_world[10]));
    } else {
        view = safe_normalize(sub3(ld3(p.camera_pos), world));
    }

    // direct_light (shade.wesl:429-521)
    const Shape shape = lobe_shape(roughness, tilt);
    const float tv = dot3(tangent, view);
    const float cos_theta_o = sqrtf(fmaxf(1.0f - tv * tv, 1e-6f));
    const f3 sigma_a = absorption_from_color(albedo, roughness);
    const Dual ds = dual_scatter(cos_theta_o, sigma_a, shape);
    f3 color = spl(0.0f);
    bool dom_left = true;
    const f3 t_n = safe_normalize(tangent), v_n = safe_normalize(view);
    for (uint32_t i = 0; i < n_lights; ++i) {
        const hg_light& L = lights[i];
        const uint32_t kind = L.kind;
        // each kind gives the incident direction, a weight and the DOM depth;
        // one BSDF evaluation serves them all
        f3 incident = spl(0.0f);
        float weight = 0.0f, depth = 0.0f;
        if (kind == HG_LIGHT_POINT || kind == HG_LIGHT_SPOT) {
            f3 to_l = sub3(ld3(L.position), world);
            float dist2 = dot3(to_l, to_l);
            incident = safe_normalize(to_l);
            float inv_r2 = 1.0f / fmaxf(L.range * L.range, 1e-8f);
            weight = range_window(dist2, inv_r2) / fmaxf(dist2, 1e-4f);
            if (kind == HG_LIGHT_SPOT) {
                float cd = dot3(mul3s(ld3(L.direction), -1.0f), incident);
                float sm = clampf(cd * L.spot[0] + L.spot[1], 0.0f, 1.0f);
                weight *= sm * sm;
            }
        } else if (kind == HG_LIGHT_DIRECTIONAL) {
            if (dom_left && (L.flags & HG_LIGHT_CASTS_SHADOWS)) {
                depth = -logf(fmaxf(dom_visibility(p, a.dom, world, beta), 1e-6f));
                dom_left = false;
            }
            incident = ld3(L.direction);
            weight = 1.0f;
        } else if (kind == HG_LIGHT_RECT) {
            f3 to_c = sub3(ld3(L.position), world);
            float dist2 = fmaxf(dot3(to_c, to_c), 1e-4f);
            incident = mul3s(to_c, rsqrtf(dist2));
            f3 normal = safe_normalize(cross3(ld3(L.up), ld3(L.right)));
            float facing = fmaxf(dot3(normal, incident), 0.0f);
            float solid = L.spot[0] * L.spot[1] * facing / dist2;
            float range2 = fmaxf(L.range * L.range, 1e-4f);
            weight = solid * range_window(dist2, 1.0f / range2);
        }
        if (weight > 0.0f) {
            f3 lobe = hair_bsdf(t_n, v_n, incident, sigma_a, shape, ds, depth);
            color = add3(color, mul3s(vmul(lobe, ld3(L.color)), weight));
        }
    }
    if (env.spec) {
        const f3 fiber_n = safe_normalize(sub3(view, mul3s(tangent, dot3(view, tangent))));
        const f3 pr = probe_radiance(env, tangent, fiber_n, view, albedo, roughness, tilt);
        color = add3(color, mul3s(pr, pixel_ao(p, low)));
    }
    color = mul3s(color, exposure);
    a.shaded[pix] = make_float4(color.x, color.y, color.z, 1.0f);
    a.shaded_depth[pix] = view_dist;
}

// Four blocks per SM (64 registers, some spilled) measured faster than three
// (80 registers): the probe's and the DOM taps' loads want the extra warps.
__global__ void __launch_bounds__(256, 4) shade_kernel(const ShadeArgs a, const EnvArgs env) {
    shade_pixel(a, a.lights, a.n_lights, a.ortho, a.exposure, env, blockIdx.x * blockDim.x + threadIdx.x,
                blockIdx.y * blockDim.y + threadIdx.y);
}

// Batched: one tile (blockDim.x x blockDim.y pixels) of one camera view per block.
__global__ void __launch_bounds__(256, 4) batch_shade_kernel(const BatchView* __restrict__ views,
                                                             const uint32_t* __restrict__ tile_prefix, uint32_t n_cam,
                                                             const hg_light* __restrict__ lights, uint32_t n_lights,
                                                             uint32_t ortho, float exposure, const EnvArgs env) {
    uint32_t lo = 0, hi = n_cam;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (tile_prefix[mid] <= blockIdx.x) lo = mid;
        else hi = mid;
    }
    const BatchView& v = views[lo];
    const uint32_t t = blockIdx.x - tile_prefix[lo];
    const uint32_t tiles_x = (v.width + blockDim.x - 1) / blockDim.x;
    shade_pixel(v, lights, n_lights, ortho, exposure, env, (t % tiles_x) * blockDim.x + threadIdx.x,
                (t / tiles_x) * blockDim.y + threadIdx.y);
}

// The learned-surrogate variant of fs: the network gives R, TT, TRT and the
// local back-scattering per pixel and light (hg_mlp.cuh); the DOM-shadowed
// light's forward spread keeps the dual-scattering statistics of
// dual_scatter.  A warp shades 32 pixels of one row and evaluates the
// network for all of them per light, so every lane takes part in each
// evaluation; pixels without hair run it on placeholder inputs.  Azimuthal
// roughness beta_n, which the Karis fit does not have, is the fibre
// roughness clamped to the trained range [0.2, 0.8].  Per-pixel work (view
// and tangent, the shadowed light's DOM depth and spread) happens before the
// light loop, so the loop holds little besides the network's fragments.
constexpr int kSurrogateWarps = 8;
constexpr size_t kSurrogateSmem = sizeof(mlp::FwdWeights) + kSurrogateWarps * sizeof(mlp::WarpIo);

// Incident direction and weight (scalar factor on the light colour) of a
// point, spot or rect light; directional lights have weight 1.
__device__ __forceinline__ float light_weight(const hg_light& L, f3 world, f3& incident) {
    const uint32_t kind = L.kind;
    if (kind == HG_LIGHT_POINT || kind == HG_LIGHT_SPOT) {
        f3 to_l = sub3(ld3(L.position), world);
        float dist2 = dot3(to_l, to_l);
        incident = safe_normalize(to_l);
        float inv_r2 = 1.0f / fmaxf(L.range * L.range, 1e-8f);
        float w = range_window(dist2, inv_r2) / fmaxf(dist2, 1e-4f);
        if (kind == HG_LIGHT_SPOT) {
            float cd = dot3(mul3s(ld3(L.direction), -1.0f), incident);
            float sm = clampf(cd * L.spot[0] + L.spot[1], 0.0f, 1.0f);
            w *= sm * sm;
        }
        return w;
    }
    if (kind == HG_LIGHT_DIRECTIONAL) {
        incident = ld3(L.direction);
        return 1.0f;
    }
    if (kind == HG_LIGHT_RECT) {
        f3 to_c = sub3(ld3(L.position), world);
        float dist2 = fmaxf(dot3(to_c, to_c), 1e-4f);
        incident = mul3s(to_c, rsqrtf(dist2));
        f3 normal = safe_normalize(cross3(ld3(L.up), ld3(L.right)));
        float facing = fmaxf(dot3(normal, incident), 0.0f);
        float solid = L.spot[0] * L.spot[1] * facing / dist2;
        float range2 = fmaxf(L.range * L.range, 1e-4f);
        return solid * range_window(dist2, 1.0f / range2);
    }
    incident = spl(0.0f);
    return 0.0f;
}

__global__ void __launch_bounds__(kSurrogateWarps * 32, 2)
    shade_surrogate_kernel(const ShadeArgs a, const __half* __restrict__ w16, const float* __restrict__ mparams,
                           const EnvArgs env) {
    extern __shared__ __align__(16) unsigned char smem[];
    mlp::FwdWeights& w = *reinterpret_cast<mlp::FwdWeights*>(smem);
    mlp::WarpIo& io = reinterpret_cast<mlp::WarpIo*>(smem + sizeof(mlp::FwdWeights))[threadIdx.x >> 5];
    mlp::load_fwd(w, w16, mparams, threadIdx.x, blockDim.x);
    __syncthreads();
    const hg_hair_params& p = a.p;
    const uint32_t width = f2u(p.screen[0]), height = f2u(p.screen[1]);
    const uint32_t tiles_x = (width + 31u) >> 5, tiles = tiles_x * ((height + 7u) >> 3);
    const uint32_t lane = threadIdx.x & 31u, row = threadIdx.x >> 5;
    // The light that receives the deep-opacity depth: the first shadow-casting
    // directional light in the kind-sorted list (shade.wesl:486-503).
    int dom_light = -1;
    for (uint32_t i = 0; i < a.n_lights; ++i)
        if (a.lights[i].kind == HG_LIGHT_DIRECTIONAL && (a.lights[i].flags & HG_LIGHT_CASTS_SHADOWS)) {
            dom_light = (int)i;
            break;
        }
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t x = (tile % tiles_x) * 32u + lane, y = (tile / tiles_x) * 8u + row;
        const bool inside = x < width && y < height;
        const uint32_t pix = y * width + x;
        unsigned long long word = 0ull;
        bool active = false;
        if (inside) {
            word = __ldg(&a.center[pix]);
            active = !is_empty(word);
            if (!active) {
                a.shaded[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                a.shaded_depth[pix] = 0.0f;
            }
        }
        if (!__any_sync(0xffffffffu, active)) continue;
        const uint32_t low = (uint32_t)word, high = (uint32_t)(word >> 32);
        const float view_dist = dequantize_depth(high >> 8u, p.screen[2], p.screen[3]);
        const f3 world = reconstruct_world(p, (int32_t)x, (int32_t)y, view_dist);
        const f3 tangent = oct_decode(high & 0xffu, low >> 24u);
        const float uvw_z = (float)((low >> 6u) & 0x3fu) / 63.0f;
        const float roughness = fmaxf(p.appearance[0] * (0.65f + 0.7f * uvw_z), 0.04f);
        const float ascale = 0.65f + 0.35f * uvw_z;
        const f3 albedo = {p.albedo[0] * ascale, p.albedo[1] * ascale, p.albedo[2] * ascale};
        f3 view;
        if (a.ortho) {
            view = safe_normalize(mk3(p.clip_from_world[2], p.clip_from_world[6], p.clip_from_world[10]));
        } else {
            view = safe_normalize(sub3(ld3(p.camera_pos), world));
        }
        const Shape shape = lobe_shape(roughness, p.appearance[1]);
        const f3 sigma_a = absorption_from_color(albedo, roughness);
        const float beta_n = clampf(roughness, 0.2f, 0.8f);
        const f3 t_n = safe_normalize(tangent), v_n = safe_normalize(view);
        const float sin_o = clampf(dot3(t_n, v_n), -1.0f, 1.0f);
        const f3 t_o = sub3(v_n, mul3s(t_n, sin_o));
        const float to2 = dot3(t_o, t_o);
        f3 color = spl(0.0f);
        float dom_direct = 1.0f;
        if (dom_light >= 0 && active) {
            const hg_light& L = a.lights[dom_light];
            const float beta = (float)(__ldg(&a.beta[pix]) & 0xffu) / 255.0f;
            const float depth = -logf(fmaxf(dom_visibility(p, a.dom, world, beta), 1e-6f));
            dom_direct = expf(-depth);
            if (depth > 1e-3f) {
                const float tv = dot3(tangent, view);
                const Dual ds = dual_scatter(sqrtf(fmaxf(1.0f - tv * tv, 1e-6f)), sigma_a, shape);
                const Geometry gm = light_geometry(t_n, v_n, ld3(L.direction));
                color = vmul(spread_term(shape, ds, gm.theta_h, depth, dom_direct), ld3(L.color));
            }
        }
        for (uint32_t i = 0; i < a.n_lights; ++i) {
            const hg_light& L = a.lights[i];
            f3 incident;
            float weight = light_weight(L, world, incident);
            if ((int)i == dom_light) weight = dom_direct;
            const bool use = active && weight > 0.0f;
            if (!__any_sync(0xffffffffu, use)) continue;
            // sin theta_i and cos phi as light_geometry computes them (the
            // network needs no angles).
            const f3 l = safe_normalize(incident);
            const float sin_i = clampf(dot3(t_n, l), -1.0f, 1.0f);
            const f3 t_i = sub3(l, mul3s(t_n, sin_i));
            const float proj = sqrtf(fmaxf(dot3(t_i, t_i) * to2, 1e-8f));
            const float cos_phi = clampf(dot3(t_i, t_o) / proj, -1.0f, 1.0f);
            float raw[10] = {sin_i, sin_o, cos_phi, sqrtf(fmaxf(1.0f - cos_phi * cos_phi, 0.0f)),
                             sigma_a.x, sigma_a.y, sigma_a.z, shape.beta.x, beta_n, kIor};
            if (!use) {
                raw[0] = raw[1] = raw[3] = 0.0f;
                raw[2] = 1.0f;
                raw[4] = raw[5] = raw[6] = 0.4f;
                raw[7] = mlp::kBetaMMid;
                raw[8] = mlp::kBetaNMid;
            }
            float xn[10], yv[12];
            mlp::normalise(raw, xn);
            mlp::forward_fast(w, io, xn, yv);
            if (use) {
                f3 lobe = {mlp::decode_fast(yv[0]) + mlp::decode_fast(yv[3]) + mlp::decode_fast(yv[6]),
                           mlp::decode_fast(yv[1]) + mlp::decode_fast(yv[4]) + mlp::decode_fast(yv[7]),
                           mlp::decode_fast(yv[2]) + mlp::decode_fast(yv[5]) + mlp::decode_fast(yv[8])};
                lobe = add3(lobe, mul3s(mk3(mlp::decode_fast(yv[9]), mlp::decode_fast(yv[10]),
                                            mlp::decode_fast(yv[11])),
                                        kDensityBack));
                color = add3(color, mul3s(vmul(lobe, ld3(L.color)), weight));
            }
        }
        if (active) {
            if (env.spec) {
                const f3 fiber_n = safe_normalize(sub3(view, mul3s(tangent, dot3(view, tangent))));
                const f3 pr = probe_radiance(env, tangent, fiber_n, view, albedo, roughness, p.appearance[1]);
                color = add3(color, mul3s(pr, pixel_ao(p, low)));
            }
            color = mul3s(color, a.exposure);
            a.shaded[pix] = make_float4(color.x, color.y, color.z, 1.0f);
            a.shaded_depth[pix] = view_dist;
        }
    }
}

// The 12 lobes R, TT, TRT, B of the Karis fit for surrogate-style inputs
// (sin_i, sin_o, cos_phi, sin_phi, sigma_a rgb, beta_m, beta_n, eta), as
// hair_bsdf and dual_scatter evaluate them; beta_n and eta do not enter the
// fit (its IOR is fixed at 1.55).
__global__ void karis_lobes_kernel(const float* __restrict__ in, uint32_t n, float tilt, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* x = in + (size_t)i * 10;
    const float sin_i = clampf(x[0], -1.0f, 1.0f), sin_o = clampf(x[1], -1.0f, 1.0f);
    const float cos_phi = clampf(x[2], -1.0f, 1.0f);
    const f3 sigma_a = {x[4], x[5], x[6]};
    const float bm = x[7];
    const Shape shape = {{tilt, -0.5f * tilt, -1.5f * tilt}, {bm, 0.5f * bm, 2.0f * bm}};
    const float theta_i = asinf(sin_i), theta_o = asinf(sin_o), theta_h = theta_i + theta_o;
    const float cos_theta_d = fmaxf(cosf(0.5f * fabsf(theta_i - theta_o)), 1e-3f);
    const Lobes l = azimuthal(cos_theta_d, cos_phi, sigma_a);
    const f3 m = gaussian3(shape.beta, sub3(spl(theta_h), shape.alpha));
    const Dual ds = dual_scatter(sqrtf(fmaxf(1.0f - sin_o * sin_o, 1e-6f)), sigma_a, shape);
    const f3 g = gaussian3(vsqrt(ds.sigma_b2), sub3(spl(theta_h), ds.delta_b));
    const f3 b = mul3s(vmul(ds.a_back, g), 2.0f / kPi);
    const f3 v[4] = {mul3s(l.r, m.x), mul3s(l.tt, m.y), mul3s(l.trt, m.z), b};
    float* o = out + (size_t)i * 12;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        o[3 * k] = v[k].x;
        o[3 * k + 1] = v[k].y;
        o[3 * k + 2] = v[k].z;
    }
}

// ---------------------------------------------------------------- surrogate on tcgen05
// Shade model 1: the surrogate with the network on the tcgen05 tensor cores
// (hg_mlp_tc.cuh).  A prepass lists the pixels with hair, so every one of the
// 128 MMA rows of a chunk is a real pixel; each warpgroup of a CTA shades its
// own chunks, one network evaluation per light.  The light loop, the DOM
// spread and the probe are those of shade_surrogate_kernel.

constexpr uint32_t kLightsPerStep = 1;

// Pixels whose centre word is not empty, appended in block order (one
// atomic per block of kHairListThreads x kHairListPer pixels; each thread
// loads its kHairListPer centre words before it looks at any); the others
// get the empty shade outputs.
constexpr uint32_t kHairListThreads = 256;
constexpr uint32_t kHairListPer = 8;  // pixels per thread

// The compact surrogate (shade model 3) replaces the per-light lobes; the one
// per-pixel computation left of the Karis model's prologue is dual_scatter,
// whose statistics only the deep-opacity-shadowed light's forward spread
// (spread_term) uses.  Within one shade call they depend on the pixel's
// 6-bit uvw.z (through roughness and albedo) and its view angle theta_o
// alone, so shade model 3 reads them from a table filled before the shade
// kernel: dual_scatter evaluated exactly at 64 uvw.z levels x kDualSteps + 1
// angles theta_o = k pi / (2 kDualSteps), linear in theta_o between them.
constexpr int kDualUz = 64;
constexpr int kDualSteps = 128;
constexpr int kDualEntries = kDualUz * (kDualSteps + 1);
constexpr int kDualVec = 6;  // float4 per entry
static_assert((size_t)kDualEntries * kDualVec == kDualTableFloat4, "hg_ctx::dual_table size");

__global__ void __launch_bounds__(256) dual_table_kernel(const hg_hair_params p, float4* __restrict__ table) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (uint32_t)kDualEntries) return;
    const uint32_t uz = e / (kDualSteps + 1), k = e % (kDualSteps + 1);
    const float uvw_z = (float)uz / 63.0f;
    const float roughness = fmaxf(p.appearance[0] * (0.65f + 0.7f * uvw_z), 0.04f);
    const float ascale = 0.65f + 0.35f * uvw_z;
    const f3 albedo = {p.albedo[0] * ascale, p.albedo[1] * ascale, p.albedo[2] * ascale};
    const Shape shape = lobe_shape(roughness, p.appearance[1]);
    const f3 sigma_a = absorption_from_color(albedo, roughness);
    const float theta = (float)k * (0.5f * kPi / (float)kDualSteps);
    const Dual d = dual_scatter(fmaxf(cosf(theta), 1e-3f), sigma_a, shape);
    float4* out = table + (size_t)e * kDualVec;
    out[0] = make_float4(d.fwd.r.x, d.fwd.r.y, d.fwd.r.z, d.a_f.x);
    out[1] = make_float4(d.fwd.tt.x, d.fwd.tt.y, d.fwd.tt.z, d.a_f.y);
    out[2] = make_float4(d.fwd.trt.x, d.fwd.trt.y, d.fwd.trt.z, d.a_f.z);
    out[3] = make_float4(d.beta_f2.x, d.beta_f2.y, d.beta_f2.z, d.sigma_b2.x);
    out[4] = make_float4(d.a_back.x, d.a_back.y, d.a_back.z, d.sigma_b2.y);
    out[5] = make_float4(d.delta_b.x, d.delta_b.y, d.delta_b.z, d.sigma_b2.z);
}

// dual_scatter of a pixel from the table: uvw.z level uz, |sin theta_o| = |t . v|.
__device__ __forceinline__ Dual dual_from_table(const float4* __restrict__ table, uint32_t uz, float sin_o_abs) {
    const float pos = asinf(fminf(sin_o_abs, 1.0f)) * ((float)kDualSteps / (0.5f * kPi));
    const int k0 = min(max((int)pos, 0), kDualSteps - 1);
    const float f = clampf(pos - (float)k0, 0.0f, 1.0f);
    const float4* e0 = table + ((size_t)uz * (kDualSteps + 1) + k0) * kDualVec;
    const float4* e1 = e0 + kDualVec;
    float4 v[kDualVec];
#pragma unroll
    for (int q = 0; q < kDualVec; ++q) {
        const float4 a = __ldg(e0 + q), b = __ldg(e1 + q);
        v[q] = make_float4(a.x + f * (b.x - a.x), a.y + f * (b.y - a.y), a.z + f * (b.z - a.z), a.w + f * (b.w - a.w));
    }
    Dual d;
    d.fwd.r = mk3(v[0].x, v[0].y, v[0].z);
    d.fwd.tt = mk3(v[1].x, v[1].y, v[1].z);
    d.fwd.trt = mk3(v[2].x, v[2].y, v[2].z);
    d.a_f = mk3(v[0].w, v[1].w, v[2].w);
    d.beta_f2 = mk3(v[3].x, v[3].y, v[3].z);
    d.a_back = mk3(v[4].x, v[4].y, v[4].z);
    d.delta_b = mk3(v[5].x, v[5].y, v[5].z);
    d.sigma_b2 = mk3(v[3].w, v[4].w, v[5].w);
    return d;
}

__global__ void __launch_bounds__(kHairListThreads) hair_list_kernel(const unsigned long long* __restrict__ center,
                                                                      uint32_t pixels, uint32_t* __restrict__ list,
                                                                      uint32_t* __restrict__ count,
                                                                      float4* __restrict__ shaded,
                                                                      float* __restrict__ shaded_depth) {
    __shared__ uint32_t warp_off[kHairListThreads / 32];
    __shared__ uint32_t block_base;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t first = blockIdx.x * (kHairListThreads * kHairListPer) + threadIdx.x;
    // every load in flight before the first use
    unsigned long long w[kHairListPer];
#pragma unroll
    for (uint32_t k = 0; k < kHairListPer; ++k) {
        const uint32_t px = first + k * kHairListThreads;
        w[k] = px < pixels ? __ldg(&center[px]) : kEmptyU64;
    }
    uint32_t mine = 0, total = 0;
    uint32_t mask[kHairListPer];
#pragma unroll
    for (uint32_t k = 0; k < kHairListPer; ++k) {
        const uint32_t px = first + k * kHairListThreads;
        const bool hair = px < pixels && !is_empty(w[k]);
        if (px < pixels && !hair) {
            shaded[px] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            shaded_depth[px] = 0.0f;
        }
        mask[k] = __ballot_sync(0xffffffffu, hair);
        mine |= hair ? 1u << k : 0u;
        total += (uint32_t)__popc(mask[k]);
    }
    if (lane == 0) warp_off[warp] = total;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t sum = 0;
        for (uint32_t v = 0; v < kHairListThreads / 32u; ++v) {
            const uint32_t c = warp_off[v];
            warp_off[v] = sum;
            sum += c;
        }
        block_base = sum ? atomicAdd(count, sum) : 0u;
    }
    __syncthreads();
    uint32_t at = block_base + warp_off[warp];
#pragma unroll
    for (uint32_t k = 0; k < kHairListPer; ++k) {
        if (mine & (1u << k)) list[at + __popc(mask[k] & ((1u << lane) - 1u))] = first + k * kHairListThreads;
        at += (uint32_t)__popc(mask[k]);
    }
}

__global__ void __launch_bounds__(mlp::tc::kThreads, 1)
    shade_tc_kernel(const ShadeArgs a, const __half* __restrict__ w16, const float* __restrict__ mparams,
                    const EnvArgs env, const uint32_t* __restrict__ list, const uint32_t* __restrict__ count,
                    uint32_t* __restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem_tc[];
    mlp::tc::Chain c = mlp::tc::setup(smem_tc, w16, mparams);
    const hg_hair_params& p = a.p;
    const uint32_t width = f2u(p.screen[0]);
    const uint32_t g = threadIdx.x >> 7;
    int dom_light = -1;
    for (uint32_t i = 0; i < a.n_lights; ++i)
        if (a.lights[i].kind == HG_LIGHT_DIRECTIONAL && (a.lights[i].flags & HG_LIGHT_CASTS_SHADOWS)) {
            dom_light = (int)i;
            break;
        }
    const uint32_t n = *count;
    const uint32_t chunks = (n + mlp::tc::kM - 1) / mlp::tc::kM;
    bool failed = false;
    for (uint32_t ch = blockIdx.x * mlp::tc::kChains + g; ch < chunks; ch += gridDim.x * mlp::tc::kChains) {
        const uint32_t idx = ch * mlp::tc::kM + c.row;
        const bool active = idx < n;
        const uint32_t pix = active ? __ldg(&list[idx]) : 0u;
        const uint32_t x = pix % width, y = pix / width;
        const unsigned long long word = active ? __ldg(&a.center[pix]) : 0ull;
        const uint32_t low = (uint32_t)word, high = (uint32_t)(word >> 32);
        const float view_dist = dequantize_depth(high >> 8u, p.screen[2], p.screen[3]);
        const f3 world = reconstruct_world(p, (int32_t)x, (int32_t)y, view_dist);
        const f3 tangent = oct_decode(high & 0xffu, low >> 24u);
        const float uvw_z = (float)((low >> 6u) & 0x3fu) / 63.0f;
        const float roughness = fmaxf(p.appearance[0] * (0.65f + 0.7f * uvw_z), 0.04f);
        const float ascale = 0.65f + 0.35f * uvw_z;
        const f3 albedo = {p.albedo[0] * ascale, p.albedo[1] * ascale, p.albedo[2] * ascale};
        f3 view;
        if (a.ortho) {
            view = safe_normalize(mk3(p.clip_from_world[2], p.clip_from_world[6], p.clip_from_world[10]));
        } else {
            view = safe_normalize(sub3(ld3(p.camera_pos), world));
        }
        const Shape shape = lobe_shape(roughness, p.appearance[1]);
        const f3 sigma_a = absorption_from_color(albedo, roughness);
        const float beta_n = clampf(roughness, 0.2f, 0.8f);
        const f3 t_n = safe_normalize(tangent), v_n = safe_normalize(view);
        const float sin_o = clampf(dot3(t_n, v_n), -1.0f, 1.0f);
        const f3 t_o = sub3(v_n, mul3s(t_n, sin_o));
        const float to2 = dot3(t_o, t_o);
        // the per-pixel network inputs (absorption, roughnesses, IOR)
        float xin[10];
        {
            const float raw[10] = {0.0f, 0.0f, 1.0f, 0.0f, sigma_a.x, sigma_a.y, sigma_a.z, shape.beta.x, beta_n, kIor};
            mlp::normalise(raw, xin);
        }
        f3 color = spl(0.0f);
        float dom_direct = 1.0f;
        if (dom_light >= 0 && active) {
            const hg_light& L = a.lights[dom_light];
            const float beta = (float)(__ldg(&a.beta[pix]) & 0xffu) / 255.0f;
            const float depth = -logf(fmaxf(dom_visibility(p, a.dom, world, beta), 1e-6f));
            dom_direct = expf(-depth);
            if (depth > 1e-3f) {
                const float tv = dot3(tangent, view);
                const Dual ds = dual_scatter(sqrtf(fmaxf(1.0f - tv * tv, 1e-6f)), sigma_a, shape);
                const Geometry gm = light_geometry(t_n, v_n, ld3(L.direction));
                color = vmul(spread_term(shape, ds, gm.theta_h, depth, dom_direct), ld3(L.color));
            }
        }
        // lights two at a time: the chain's two evaluations
        for (uint32_t i = 0; i < a.n_lights; i += kLightsPerStep) {
            const bool two = kLightsPerStep == 2 && i + 1 < a.n_lights;
            float weight[2] = {0.0f, 0.0f};
            for (uint32_t e = 0; e < (two ? 2u : 1u); ++e) {
                const hg_light& L = a.lights[i + e];
                f3 incident;
                float w = light_weight(L, world, incident);
                if ((int)(i + e) == dom_light) w = dom_direct;
                const bool use = active && w > 0.0f;
                weight[e] = use ? w : 0.0f;
                const f3 l = safe_normalize(incident);
                const float sin_i = clampf(dot3(t_n, l), -1.0f, 1.0f);
                const f3 t_i = sub3(l, mul3s(t_n, sin_i));
                const float proj = sqrtf(fmaxf(dot3(t_i, t_i) * to2, 1e-8f));
                const float cos_phi = clampf(dot3(t_i, t_o) / proj, -1.0f, 1.0f);
                xin[0] = use ? sin_i : 0.0f;
                xin[1] = use ? sin_o : 0.0f;
                xin[2] = use ? cos_phi : 1.0f;
                xin[3] = use ? sqrtf(fmaxf(1.0f - cos_phi * cos_phi, 0.0f)) : 0.0f;
                mlp::tc::write_input_row(c, e, xin);
            }
            float yv[2][12];
            if (!mlp::tc::forward2(c, two, yv[0], yv[1])) {
                failed = true;
                break;
            }
            for (uint32_t e = 0; e < (two ? 2u : 1u); ++e) {
                if (!(weight[e] > 0.0f)) continue;
                const float* q = yv[e];
                f3 lobe = {mlp::decode_fast(q[0]) + mlp::decode_fast(q[3]) + mlp::decode_fast(q[6]),
                           mlp::decode_fast(q[1]) + mlp::decode_fast(q[4]) + mlp::decode_fast(q[7]),
                           mlp::decode_fast(q[2]) + mlp::decode_fast(q[5]) + mlp::decode_fast(q[8])};
                lobe = add3(lobe, mul3s(mk3(mlp::decode_fast(q[9]), mlp::decode_fast(q[10]), mlp::decode_fast(q[11])),
                                        kDensityBack));
                color = add3(color, mul3s(vmul(lobe, ld3(a.lights[i + e].color)), weight[e]));
            }
        }
        if (failed) break;
        if (active) {
            if (env.spec) {
                const f3 fiber_n = safe_normalize(sub3(view, mul3s(tangent, dot3(view, tangent))));
                const f3 pr = probe_radiance(env, tangent, fiber_n, view, albedo, roughness, p.appearance[1]);
                color = add3(color, mul3s(pr, pixel_ao(p, low)));
            }
            color = mul3s(color, a.exposure);
            a.shaded[pix] = make_float4(color.x, color.y, color.z, 1.0f);
            a.shaded_depth[pix] = view_dist;
        }
    }
    if (failed && c.row == 0) atomicOr(err, mlp::tc::kErrTimeout);
    mlp::tc::teardown(smem_tc, c, failed);
}

// ---------------------------------------------------------------- compact surrogate
// Shade model 3: the compact 2 x 32 network (hg_mlp_small.cuh), whose three
// outputs are the per-light BSDF rgb, on mma.sync.  The hair-pixel list of
// shade model 1 fills every lane: a warp shades 32 listed pixels and
// evaluates the network for all of them once per light.
//
// Layout choices that keep the light loop short:
// * Lane L = 4g + t puts its pixel in network row g + 8t, and the output
//   layer's rows are duplicated in shared memory so that every lane's
//   C-fragment columns 2t, 2t+1, 8+2t are red, green, blue (9+2t is zero):
//   each lane then holds the three outputs of all four rows g + 8k of its
//   fragments and keeps row g + 8t, its own pixel.  No shuffles, three
//   exponentials per lane and light.
// * Each pixel's inputs sit in shared row L (row stride 13 words: stores
//   and the permuted fragment loads are both free of bank conflicts); the
//   per-pixel inputs (sin theta_o, absorption, roughnesses, IOR) are written
//   once per pixel, per light only sin theta_i, cos phi and sin phi.
// * Biases are stored as the accumulator quads {b(2t), b(2t+1), b(2t),
//   b(2t+1)} and enter the first MMA of a layer as its C operand.
constexpr int kCompactWarps = 8;
constexpr int kXPad = 26;  // halves per input row

// A light with its per-light constants worked out once per block.
struct CompactLight {
    float4 pos;     // position, 1 / max(range^2, 1e-8)
    float4 dir;     // direction (normalized for directional lights), kind as bits
    float4 color;   // colour, spot scale
    float4 normal;  // rect normal, spot offset
    float4 rect;    // rect area (spot[0] * spot[1]), 1 / max(range^2, 1e-4), flags as bits, 0
};

struct CompactSmem {
    __half w1[mlps::kHid][mlps::kPadIn];
    __half w2[mlps::kHid][mlps::kPadHid];
    __half w3[mlps::kOut][mlps::kPadHid];  // rows duplicated, see above
    float4 bq1[4][4], bq2[4][4], bq3[2][4];  // [n-tile][t]
    __half x[kCompactWarps][32][kXPad];
    CompactLight lights[HG_MAX_LIGHTS];
};

__device__ __forceinline__ CompactLight compact_light(const hg_light& L) {
    CompactLight c;
    const f3 dir = L.kind == HG_LIGHT_DIRECTIONAL ? safe_normalize(ld3(L.direction)) : ld3(L.direction);
    const f3 nrm = safe_normalize(cross3(ld3(L.up), ld3(L.right)));
    c.pos = make_float4(L.position[0], L.position[1], L.position[2], 1.0f / fmaxf(L.range * L.range, 1e-8f));
    c.dir = make_float4(dir.x, dir.y, dir.z, __uint_as_float(L.kind));
    c.color = make_float4(L.color[0], L.color[1], L.color[2], L.spot[0]);
    c.normal = make_float4(nrm.x, nrm.y, nrm.z, L.spot[1]);
    c.rect = make_float4(L.spot[0] * L.spot[1], 1.0f / fmaxf(L.range * L.range, 1e-4f), __uint_as_float(L.flags), 0.0f);
    return c;
}

// light_weight with the per-light constants; l is the unit direction to the light.
__device__ __forceinline__ float compact_weight(const CompactLight& c, f3 world, f3& l) {
    const uint32_t kind = __float_as_uint(c.dir.w);
    if (kind == HG_LIGHT_DIRECTIONAL) {
        l = mk3(c.dir.x, c.dir.y, c.dir.z);
        return 1.0f;
    }
    const f3 to_l = sub3(mk3(c.pos.x, c.pos.y, c.pos.z), world);
    if (kind == HG_LIGHT_POINT || kind == HG_LIGHT_SPOT) {
        const float dist2 = dot3(to_l, to_l);
        l = safe_normalize(to_l);
        float w = range_window(dist2, c.pos.w) / fmaxf(dist2, 1e-4f);
        if (kind == HG_LIGHT_SPOT) {
            const float cd = -dot3(mk3(c.dir.x, c.dir.y, c.dir.z), l);
            const float sm = clampf(cd * c.color.w + c.normal.w, 0.0f, 1.0f);
            w *= sm * sm;
        }
        return w;
    }
    if (kind == HG_LIGHT_RECT) {
        const float dist2 = fmaxf(dot3(to_l, to_l), 1e-4f);
        l = mul3s(to_l, rsqrtf(dist2));
        const float facing = fmaxf(dot3(mk3(c.normal.x, c.normal.y, c.normal.z), l), 0.0f);
        return c.rect.x * facing / dist2 * range_window(dist2, c.rect.y);
    }
    l = mk3(0.0f, 1.0f, 0.0f);
    return 0.0f;
}

// Output row of the network in physical column pc of the duplicated layer:
// red in even columns 0..6, green in odd columns 1..7, blue in even columns
// 8..14, zero (padding row 15) in odd columns 9..15.
__device__ __forceinline__ int compact_out_row(int pc) {
    if (pc < 8) return pc & 1;
    return (pc & 1) ? mlps::kOut - 1 : 2;
}

__device__ __forceinline__ void st_h2(__half* p, float lo, float hi) {
    *reinterpret_cast<uint32_t*>(p) = mlp::pack_h2(lo, hi);
}

// D = A * B + C with a separate C (the bias quad).
__device__ __forceinline__ void mma_c(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1, const float4& c) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%10,%11,%12,%13};\n"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(c.x), "f"(c.y), "f"(c.z), "f"(c.w));
}

// One layer for MT m-tiles: acc[mt][nt] = bias + A[mt] * W^T, N = 8 NT
// outputs, K = 16 KT inputs.
template <int MT, int NT, int KT, int PAD>
__device__ __forceinline__ void compact_layer(float acc[][NT][4], const uint32_t a[][KT][4], const __half (*w)[PAD],
                                              const float4 (*bq)[4], int lane) {
    const int t = lane & 3, mat = lane >> 3, r = lane & 7;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            uint32_t b[4];
            mlp::ldsm_x4(b, &w[(nt + (mat >> 1)) * 8 + r][kt * 16 + (mat & 1) * 8]);
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                if (kt == 0) {
                    mma_c(acc[mt][nt], a[mt][0], b[0], b[1], bq[nt][t]);
                    mma_c(acc[mt][nt + 1], a[mt][0], b[2], b[3], bq[nt + 1][t]);
                } else {
                    mlp::mma(acc[mt][nt], a[mt][kt], b[0], b[1]);
                    mlp::mma(acc[mt][nt + 1], a[mt][kt], b[2], b[3]);
                }
            }
        }
    }
}

// C fragments of a 32-wide layer -> ReLU -> FP16 A fragments of the next.
template <int MT>
__device__ __forceinline__ void compact_relu(const float acc[][4][4], uint32_t a[][2][4]) {
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            const float* lo = acc[mt][2 * kt];
            const float* hi = acc[mt][2 * kt + 1];
            a[mt][kt][0] = mlp::pack_relu(lo[0], lo[1]);
            a[mt][kt][1] = mlp::pack_relu(lo[2], lo[3]);
            a[mt][kt][2] = mlp::pack_relu(hi[0], hi[1]);
            a[mt][kt][3] = mlp::pack_relu(hi[2], hi[3]);
        }
}

// m-tiles evaluated together (2) or one after the other (1): one after the
// other leaves room for three blocks per SM.
constexpr int kCompactTiles = 1;
// Resident blocks per SM of the compact shade kernel.
constexpr int kCompactBlocks = 4;

__device__ __forceinline__ float4 bias_quad(const float* b, int nt, int t) {
    const float lo = b[nt * 8 + 2 * t], hi = b[nt * 8 + 2 * t + 1];
    return make_float4(lo, hi, lo, hi);
}

__global__ void __launch_bounds__(kCompactWarps * 32, kCompactBlocks)
    shade_compact_kernel(const ShadeArgs a, const __half* __restrict__ w16, const float* __restrict__ mparams,
                         const EnvArgs env, const uint32_t* __restrict__ list, const uint32_t* __restrict__ count,
                         const float4* __restrict__ dual_table) {
    __shared__ __align__(16) CompactSmem sm;
    {
        const int tid = threadIdx.x, nth = blockDim.x;
        mlp::copy_rows<mlps::kPadIn>(sm.w1, w16 + mlps::kW1, mlps::kHid, mlps::kIn, tid, nth);
        mlp::copy_rows<mlps::kPadHid>(sm.w2, w16 + mlps::kW2, mlps::kHid, mlps::kHid, tid, nth);
        for (int i = tid; i < mlps::kOut * (mlps::kHid / 8); i += nth) {
            const int pc = i / (mlps::kHid / 8), c = (i % (mlps::kHid / 8)) * 8;
            *reinterpret_cast<uint4*>(&sm.w3[pc][c]) =
                __ldg(reinterpret_cast<const uint4*>(w16 + mlps::kW3 + compact_out_row(pc) * mlps::kHid + c));
        }
        for (int i = tid; i < 16; i += nth) {
            const int nt = i >> 2, tt = i & 3;
            sm.bq1[nt][tt] = bias_quad(mparams + mlps::kB1, nt, tt);
            sm.bq2[nt][tt] = bias_quad(mparams + mlps::kB2, nt, tt);
            if (nt < 2) {
                const float lo = mparams[mlps::kB3 + compact_out_row(nt * 8 + 2 * tt)];
                const float hi = mparams[mlps::kB3 + compact_out_row(nt * 8 + 2 * tt + 1)];
                sm.bq3[nt][tt] = make_float4(lo, hi, lo, hi);
            }
        }
        for (uint32_t i = tid; i < a.n_lights; i += nth) sm.lights[i] = compact_light(a.lights[i]);
    }
    __syncthreads();
    // Everything above reads only the weights and lights; the hair list
    // comes from the kernel before (programmatic dependent launch).
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const hg_hair_params& p = a.p;
    const uint32_t width = f2u(p.screen[0]);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int g = (int)(lane >> 2), t = (int)(lane & 3u);
    __half(*xr)[kXPad] = sm.x[warp];
    // The light that receives the deep-opacity depth (shade.wesl:486-503).
    int dom_light = -1;
    for (uint32_t i = 0; i < a.n_lights; ++i)
        if (a.lights[i].kind == HG_LIGHT_DIRECTIONAL && (a.lights[i].flags & HG_LIGHT_CASTS_SHADOWS)) {
            dom_light = (int)i;
            break;
        }
    const uint32_t n = *count;
    const uint32_t chunks = (n + 31u) >> 5;
    const uint32_t stride = gridDim.x * kCompactWarps;
    // Loads run ahead of the shading: list entries two chunks, centre and
    // beta words one chunk.
    constexpr uint32_t kNone = 0xffffffffu;
    auto list_at = [&](uint32_t c) -> uint32_t {
        return c < chunks && c * 32u + lane < n ? __ldg(&list[c * 32u + lane]) : kNone;
    };
    // The block's warps take chunks in lockstep (every warp runs the same
    // number of iterations) and meet at a barrier before the probe: warps
    // spread over the prologue, the light loop and the probe at once ran more
    // code than the instruction caches hold (8 % slower with the probe on).
    const uint32_t first = blockIdx.x * kCompactWarps;
    uint32_t ch = first + warp;
    uint32_t pix_next = list_at(ch), pix_after = list_at(ch + stride);
    unsigned long long word_next = pix_next != kNone ? __ldg(&a.center[pix_next]) : 0ull;
    uint32_t beta_next = pix_next != kNone ? __ldg(&a.beta[pix_next]) : 0u;
    for (uint32_t block_ch = first; block_ch < chunks; block_ch += stride, ch += stride) {
        const bool active = pix_next != kNone;
        const uint32_t pix = active ? pix_next : 0u;
        const unsigned long long word = word_next;
        const uint32_t beta_word = beta_next;
        word_next = pix_after != kNone ? __ldg(&a.center[pix_after]) : 0ull;
        beta_next = pix_after != kNone ? __ldg(&a.beta[pix_after]) : 0u;
        pix_next = pix_after;
        pix_after = list_at(ch + 2 * stride);
        const uint32_t x = pix % width, y = pix / width;
        const uint32_t low = (uint32_t)word, high = (uint32_t)(word >> 32);
        const float view_dist = dequantize_depth(high >> 8u, p.screen[2], p.screen[3]);
        const f3 world = reconstruct_world(p, (int32_t)x, (int32_t)y, view_dist);
        const f3 tangent = oct_decode(high & 0xffu, low >> 24u);
        const float uvw_z = (float)((low >> 6u) & 0x3fu) / 63.0f;
        const float roughness = fmaxf(p.appearance[0] * (0.65f + 0.7f * uvw_z), 0.04f);
        const float ascale = 0.65f + 0.35f * uvw_z;
        const f3 albedo = {p.albedo[0] * ascale, p.albedo[1] * ascale, p.albedo[2] * ascale};
        f3 view;
        if (a.ortho) {
            view = safe_normalize(mk3(p.clip_from_world[2], p.clip_from_world[6], p.clip_from_world[10]));
        } else {
            view = safe_normalize(sub3(ld3(p.camera_pos), world));
        }
        const Shape shape = lobe_shape(roughness, p.appearance[1]);
        const f3 sigma_a = absorption_from_color(albedo, roughness);
        const f3 t_n = safe_normalize(tangent), v_n = safe_normalize(view);
        const float sin_o = clampf(dot3(t_n, v_n), -1.0f, 1.0f);
        const f3 t_o = sub3(v_n, mul3s(t_n, sin_o));
        const float to2 = dot3(t_o, t_o);
        // this pixel's row: the per-pixel inputs, columns 0, 2, 3 filled per light
        {
            const float raw[10] = {0.0f, sin_o, 1.0f, 0.0f, sigma_a.x, sigma_a.y, sigma_a.z, shape.beta.x,
                                   clampf(roughness, 0.2f, 0.8f), kIor};
            float xin[10];
            mlp::normalise(raw, xin);
            __syncwarp();
#pragma unroll
            for (int c = 0; c < 10; c += 2) st_h2(&xr[lane][c], xin[c], xin[c + 1]);
#pragma unroll
            for (int c = 10; c < mlps::kIn; c += 2) st_h2(&xr[lane][c], 0.0f, 0.0f);
            __syncwarp();
        }
        f3 color = spl(0.0f);
        float dom_direct = 1.0f;
        if (dom_light >= 0 && active) {
            const CompactLight& L = sm.lights[dom_light];
            const float beta = (float)(beta_word & 0xffu) / 255.0f;
            const float depth = -logf(fmaxf(dom_visibility(p, a.dom, world, beta), 1e-6f));
            dom_direct = expf(-depth);
            if (depth > 1e-3f) {
                const Dual ds = dual_from_table(dual_table, (low >> 6u) & 0x3fu, fabsf(dot3(tangent, view)));
                const Geometry gm = light_geometry(t_n, v_n, mk3(L.dir.x, L.dir.y, L.dir.z));
                color = vmul(spread_term(shape, ds, gm.theta_h, depth, dom_direct),
                             mk3(L.color.x, L.color.y, L.color.z));
            }
        }
        for (uint32_t i = 0; i < a.n_lights; ++i) {
            const CompactLight& L = sm.lights[i];
            // unit direction to the light (normalized once, where the
            // reference normalizes the already unit vector a second time)
            f3 l;
            float weight = compact_weight(L, world, l);
            if ((int)i == dom_light) weight = dom_direct;
            const bool use = active && weight > 0.0f;
            if (!__any_sync(0xffffffffu, use)) continue;
            // sin theta_i and cos phi as light_geometry computes them
            const float sin_i = clampf(dot3(t_n, l), -1.0f, 1.0f);
            const f3 t_i = sub3(l, mul3s(t_n, sin_i));
            const float cos_phi = clampf(dot3(t_i, t_o) * rsqrtf(fmaxf(dot3(t_i, t_i) * to2, 1e-8f)), -1.0f, 1.0f);
            __syncwarp();
            st_h2(&xr[lane][0], sin_i, sin_o);
            st_h2(&xr[lane][2], cos_phi, sqrtf(fmaxf(1.0f - cos_phi * cos_phi, 0.0f)));
            __syncwarp();
            // Network row g + 8k holds the pixel of lane 4g + k, so this lane's
            // own row is g + 8t: m-tile t >> 1, half t & 1 of its fragments.
            // Columns 8..15 (per-pixel inputs) are reloaded per light rather
            // than held, which keeps the kernel within 80 registers.
            float yr = 0.0f, yg = 0.0f, yb = 0.0f;
#pragma unroll
            for (int m0 = 0; m0 < 2; m0 += kCompactTiles) {
                uint32_t a0[kCompactTiles][1][4];
#pragma unroll
                for (int q = 0; q < kCompactTiles; ++q) {
                    const int mt = m0 + q;
                    a0[q][0][0] = mlp::ld32(&xr[4 * g + 2 * mt][2 * t]);
                    a0[q][0][1] = mlp::ld32(&xr[4 * g + 2 * mt + 1][2 * t]);
                    a0[q][0][2] = mlp::ld32(&xr[4 * g + 2 * mt][8 + 2 * t]);
                    a0[q][0][3] = mlp::ld32(&xr[4 * g + 2 * mt + 1][8 + 2 * t]);
                }
                float acc[kCompactTiles][4][4];
                uint32_t ah[kCompactTiles][2][4];
                compact_layer<kCompactTiles, 4, 1, mlps::kPadIn>(acc, a0, sm.w1, sm.bq1, (int)lane);
                compact_relu<kCompactTiles>(acc, ah);
                compact_layer<kCompactTiles, 4, 2, mlps::kPadHid>(acc, ah, sm.w2, sm.bq2, (int)lane);
                compact_relu<kCompactTiles>(acc, ah);
                float out[kCompactTiles][2][4];
                compact_layer<kCompactTiles, 2, 2, mlps::kPadHid>(out, ah, sm.w3, sm.bq3, (int)lane);
#pragma unroll
                for (int q = 0; q < kCompactTiles; ++q)
                    if ((t >> 1) == m0 + q) {
                        const bool odd = (t & 1) != 0;  // selects, not a dynamic index (no local memory)
                        yr = odd ? out[q][0][2] : out[q][0][0];
                        yg = odd ? out[q][0][3] : out[q][0][1];
                        yb = odd ? out[q][1][2] : out[q][1][0];
                    }
            }
            const f3 bsdf = {mlp::decode_fast(yr), mlp::decode_fast(yg), mlp::decode_fast(yb)};
            if (use) color = add3(color, mul3s(vmul(bsdf, mk3(L.color.x, L.color.y, L.color.z)), weight));
        }
        __syncthreads();
        if (active) {
            if (env.spec) {
                // the probe's inputs again from the centre word (fewer registers live across the light loop)
                const uint32_t lw = (uint32_t)word, hw = (uint32_t)(word >> 32);
                const f3 tg = oct_decode(hw & 0xffu, lw >> 24u);
                const float uz = (float)((lw >> 6u) & 0x3fu) / 63.0f;
                const float rough = fmaxf(p.appearance[0] * (0.65f + 0.7f * uz), 0.04f);
                const float as = 0.65f + 0.35f * uz;
                const f3 alb = {p.albedo[0] * as, p.albedo[1] * as, p.albedo[2] * as};
                f3 vw;
                if (a.ortho) {
                    vw = safe_normalize(mk3(p.clip_from_world[2], p.clip_from_world[6], p.clip_from_world[10]));
                } else {
                    vw = safe_normalize(sub3(ld3(p.camera_pos), world));
                }
                const f3 fiber_n = safe_normalize(sub3(vw, mul3s(tg, dot3(vw, tg))));
                const f3 pr = probe_radiance(env, tg, fiber_n, vw, alb, rough, p.appearance[1]);
                color = add3(color, mul3s(pr, pixel_ao(p, lw)));
            }
            color = mul3s(color, a.exposure);
            a.shaded[pix] = make_float4(color.x, color.y, color.z, 1.0f);
            a.shaded_depth[pix] = dequantize_depth((uint32_t)(word >> 40), p.screen[2], p.screen[3]);
        }
    }
}

// The dual-scattering table of shade model 3 for the material of p (albedo,
// roughness, tilt), refilled only when that material differs from the one
// it holds; the refill is ordered on the stream before the shade kernel.
cudaError_t ensure_dual_table(hg_ctx* ctx, const hg_hair_params& p) {
    hg_dual_table& d = *ctx->dual_table;
    const float key[5] = {p.albedo[0], p.albedo[1], p.albedo[2], p.appearance[0], p.appearance[1]};
    if (d.valid && std::memcmp(d.key, key, sizeof(key)) == 0) return cudaSuccess;
    d.valid = false;
    dual_table_kernel<<<(kDualEntries + 255) / 256, 256, 0, ctx->stream>>>(p, d.table);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    std::memcpy(d.key, key, sizeof(key));
    d.valid = true;
    return cudaSuccess;
}

// The hair-pixel list of shade models 1 and 3 (and the empty pixels' outputs).
cudaError_t launch_hair_list(hg_ctx* ctx) {
    const uint32_t pixels = ctx->width * ctx->height;
    cudaError_t e = cudaMemsetAsync(ctx->hair_count, 0, sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) return e;
    const uint32_t per_block = kHairListThreads * kHairListPer;
    hair_list_kernel<<<(pixels + per_block - 1) / per_block, kHairListThreads, 0, ctx->stream>>>(
        ctx->center, pixels, ctx->hair_list, ctx->hair_count, ctx->shaded, ctx->shaded_depth);
    return cudaGetLastError();
}

std::mutex g_surrogate_attr_mutex;
int g_surrogate_per_sm[64] = {};  // resident blocks per SM, 0 until the attribute is set
bool g_tc_attr[64] = {};

}  // namespace

EnvArgs env_args(const hg_ctx* ctx) {
    EnvArgs e;
    e.spec = ctx->env_spec;
    e.diff = ctx->env_diff;
    e.spec_size = ctx->env_spec_size;
    e.spec_levels = ctx->env_spec_levels;
    e.diff_size = ctx->env_diff_size;
    e.diff_levels = ctx->env_diff_levels;
    for (int i = 0; i < 4; ++i) e.rot[i] = ctx->env_rot[i];
    e.intensity = ctx->env_intensity;
    if (!e.diff) e.spec = nullptr;
    return e;
}

cudaError_t ensure_shade_setup(int device) {
    static std::mutex mutex;
    static bool ready[64] = {};
    std::lock_guard<std::mutex> lock(mutex);
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (ready[device]) return cudaSuccess;
    ScatterAngle t[2 * kScatterSteps];
    const double pi = 3.14159265358979323846;
    for (int half = 0; half < 2; ++half)
        for (int i = 0; i < kScatterSteps; ++i) {
            const double u = (i + 0.5) / kScatterSteps;
            const double c = std::cos((half + u) * 0.5 * pi);
            ScatterAngle& g = t[half * kScatterSteps + i];
            g.cos_phi = (float)c;
            g.cos_half_phi = (float)std::sqrt(std::min(std::max(0.5 + 0.5 * c, 0.0), 1.0));
            g.k_tt = (float)std::exp(-3.65 * c - 3.98);
            g.k_trt = (float)std::exp(17.0 * c - 16.78);
        }
    cudaError_t e = cudaMemcpyToSymbol(c_scatter, t, sizeof(t));
    if (e == cudaSuccess) ready[device] = true;
    return e;
}

cudaError_t launch_shade(hg_ctx* ctx, const hg_hair_params& p, uint32_t n_lights, uint32_t ortho, float exposure,
                         uint32_t model) {
    const EnvArgs env = env_args(ctx);
    ShadeArgs a;
    a.p = p;
    a.center = ctx->center;
    a.beta = ctx->beta;
    a.dom = ctx->dom;
    a.lights = ctx->lights;
    a.shaded = ctx->shaded;
    a.shaded_depth = ctx->shaded_depth;
    a.n_lights = n_lights;
    a.ortho = ortho;
    a.exposure = exposure;
    if (model == 1u) {
        {
            std::lock_guard<std::mutex> lock(g_surrogate_attr_mutex);
            if (ctx->device < 0 || ctx->device >= 64) return cudaErrorInvalidDevice;
            if (!g_tc_attr[ctx->device]) {
                cudaError_t e = cudaFuncSetAttribute(shade_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)mlp::tc::kSmemBytes);
                if (e != cudaSuccess) return e;
                g_tc_attr[ctx->device] = true;
            }
        }
        cudaError_t e = launch_hair_list(ctx);
        if (e != cudaSuccess) return e;
        // one CTA per SM: it holds all 512 TMEM columns and most of the shared memory
        shade_tc_kernel<<<ctx->sm_count, mlp::tc::kThreads, mlp::tc::kSmemBytes, ctx->stream>>>(
            a, reinterpret_cast<const __half*>(ctx->surrogate->w16), ctx->surrogate->params, env, ctx->hair_list,
            ctx->hair_count, ctx->err);
        return cudaGetLastError();
    }
    if (model == 2u) {
        int per_sm = 0;
        {
            std::lock_guard<std::mutex> lock(g_surrogate_attr_mutex);
            if (ctx->device < 0 || ctx->device >= 64) return cudaErrorInvalidDevice;
            if (g_surrogate_per_sm[ctx->device] == 0) {
                cudaError_t e = cudaFuncSetAttribute(shade_surrogate_kernel,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSurrogateSmem);
                if (e == cudaSuccess)
                    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, shade_surrogate_kernel,
                                                                      kSurrogateWarps * 32, kSurrogateSmem);
                if (e != cudaSuccess) return e;
                g_surrogate_per_sm[ctx->device] = per_sm > 0 ? per_sm : 1;
            }
            per_sm = g_surrogate_per_sm[ctx->device];
        }
        const uint32_t tiles = ((ctx->width + 31u) / 32u) * ((ctx->height + 7u) / 8u);
        uint32_t blocks = (uint32_t)ctx->sm_count * (uint32_t)per_sm;
        if (blocks > tiles) blocks = tiles;
        shade_surrogate_kernel<<<blocks, kSurrogateWarps * 32, kSurrogateSmem, ctx->stream>>>(
            a, reinterpret_cast<const __half*>(ctx->surrogate->w16), ctx->surrogate->params, env);
        return cudaGetLastError();
    }
    if (model == 3u) {
        const uint32_t pixels = ctx->width * ctx->height;
        cudaError_t e = ensure_dual_table(ctx, p);
        if (e != cudaSuccess) return e;
        if ((e = launch_hair_list(ctx)) != cudaSuccess) return e;
        // kCompactBlocks resident blocks per SM (the kernel's launch bounds), grid-striding over 32-pixel chunks
        uint32_t blocks = (uint32_t)ctx->sm_count * (uint32_t)kCompactBlocks;
        const uint32_t max_chunks = (pixels + 31u) / 32u;
        const uint32_t needed = (max_chunks + kCompactWarps - 1) / kCompactWarps;
        if (blocks > needed) blocks = needed;
        // Programmatic dependent launch: the kernel's blocks start as the list
        // pass's blocks retire and load weights and lights before they wait
        // for the list.  (Letting the list pass trigger its dependents early
        // was slower: the waiting blocks take the SM slots the pass needs.)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks);
        cfg.blockDim = dim3(kCompactWarps * 32);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = ctx->stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, shade_compact_kernel, a, reinterpret_cast<const __half*>(ctx->surrogate->w16),
                                  static_cast<const float*>(ctx->surrogate->params), env,
                                  static_cast<const uint32_t*>(ctx->hair_list),
                                  static_cast<const uint32_t*>(ctx->hair_count),
                                  static_cast<const float4*>(ctx->dual_table->table));
    }
    dim3 block(32, 8);
    dim3 grid((ctx->width + 31) / 32, (ctx->height + 7) / 8);
    shade_kernel<<<grid, block, 0, ctx->stream>>>(a, env);
    return cudaGetLastError();
}

cudaError_t launch_batch_shade(hg_ctx* ctx, const BatchDev& b) {
    if (!b.total_tiles) return cudaSuccess;
    dim3 block(b.tile_w, b.tile_h);
    batch_shade_kernel<<<b.total_tiles, block, 0, ctx->stream>>>(b.views, b.tile_prefix, b.n_cam, b.lights,
                                                                  b.n_lights, b.ortho, b.exposure, env_args(ctx));
    return cudaGetLastError();
}

cudaError_t launch_karis_lobes(hg_ctx* ctx, const float* inputs, uint32_t n, float tilt, float* lobes) {
    karis_lobes_kernel<<<(n + 255u) / 256u, 256, 0, ctx->stream>>>(inputs, n, tilt, lobes);
    return cudaGetLastError();
}

}  // namespace hg
