// Hair-mesh baker: explicit strands -> bundle cages (host code).
//
// Restates bake_hair_mesh (src/bake.rs:89-213) for grooms without a scalp:
// cluster roots in a 3-D grid, absorb sparse clusters, split each cluster
// until its cage is coherent, fit 16 layer frames, splat style residuals,
// derive corner tangents and bake ambient occlusion.  Clusters are split in
// parallel (OpenMP) and concatenated in cluster order, so the output does not
// depend on the thread count.
#include "../../include/hairgb_bake.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace {

constexpr size_t kLayers = HG_LAYER_COUNT;
constexpr uint32_t kStyleU = 8, kStyleV = 8, kStyleW = 16;
constexpr uint32_t kStyleTexels = kStyleU * kStyleV * kStyleW;
// src/bake.rs:17-31
constexpr size_t kMinStrandsPerBundle = 8;
constexpr float kTargetStrandsPerCell = 180.0f;
constexpr float kMaxQuadGap = 5.0f;
constexpr float kMaxStyleStddev = 2.0f;
constexpr float kMaxMemberError = 4.0f;
constexpr int kAoRays = 8;
constexpr float kAoReach = 8.0f;
constexpr float kAoRadius = 0.45f;
constexpr float kAoMinT = 0.75f;

struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    V3 operator+(V3 o) const { return {x + o.x, y + o.y, z + o.z}; }
    V3 operator-(V3 o) const { return {x - o.x, y - o.y, z - o.z}; }
    V3 operator*(float s) const { return {x * s, y * s, z * s}; }
    V3 operator/(float s) const { return {x / s, y / s, z / s}; }
    V3 operator-() const { return {-x, -y, -z}; }
    V3& operator+=(V3 o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator-=(V3 o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float len2(V3 a) { return dot(a, a); }
inline float len(V3 a) { return std::sqrt(len2(a)); }
inline float dist(V3 a, V3 b) { return len(a - b); }
inline V3 vmin(V3 a, V3 b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
inline V3 lerp(V3 a, V3 b, float t) { return a + (b - a) * t; }
inline V3 normalize_or(V3 v, V3 fallback) {
    float r = 1.0f / len(v);
    if (std::isfinite(r) && r > 0.0f) return v * r;
    return fallback;
}
const V3 kX(1, 0, 0), kY(0, 1, 0), kZ(0, 0, 1);

struct V2 { float x = 0, y = 0; };
inline V2 clamp01(V2 a) { return {std::clamp(a.x, 0.0f, 1.0f), std::clamp(a.y, 0.0f, 1.0f)}; }

// Symmetric 3x3 as columns.
struct M3 {
    V3 c[3];
    V3 mul(V3 v) const { return c[0] * v.x + c[1] * v.y + c[2] * v.z; }
};

struct Strands {
    const V3* points;
    uint32_t n_points;
    std::vector<std::pair<uint32_t, uint32_t>> strands;  // (first, count)
};

using Samples = std::array<V3, kLayers>;

// src/bake.rs:1344-1350
V3 average(const std::vector<V3>& pts) {
    V3 acc;
    for (auto& p : pts) acc += p;
    return acc / (float)std::max<size_t>(pts.size(), 1);
}

// src/bake.rs:1368-1390
V3 dominant_axis(const M3& cov, V3 seed) {
    V3 v = normalize_or(seed, kX);
    for (int i = 0; i < 24; ++i) {
        V3 next = cov.mul(v);
        if (len2(next) < 1e-12f) break;
        v = next * (1.0f / len(next));
    }
    return v;
}
M3 deflate(const M3& cov, V3 axis) {
    float lambda = dot(axis, cov.mul(axis));
    M3 r;
    for (int j = 0; j < 3; ++j) r.c[j] = cov.c[j] - axis * (axis[j] * lambda);
    return r;
}

// src/bake.rs:1352-1366
void plane_axes(const std::vector<V3>& pts, V3& mean, V3& au, V3& av) {
    mean = average(pts);
    M3 cov;
    for (auto& p : pts) {
        V3 d = p - mean;
        cov.c[0] += d * d.x;
        cov.c[1] += d * d.y;
        cov.c[2] += d * d.z;
    }
    au = dominant_axis(cov, kX);
    M3 def = deflate(cov, au);
    av = dominant_axis(def, kY);
    if (std::fabs(dot(au, av)) > 0.99f) av = normalize_or(cross(au, kY), kX);
    av = av * (1.0f / len(av));
}

// src/bake.rs:625-681
struct Frame {
    V3 mean, axis_u, axis_v;
    float min_u = 0, max_u = 0, min_v = 0, max_v = 0;
    float width_u() const { return max_u - min_u; }
    float width_v() const { return max_v - min_v; }
    std::array<V3, 4> quad() const {
        V3 u0 = axis_u * min_u, u1 = axis_u * max_u, v0 = axis_v * min_v, v1 = axis_v * max_v;
        return {mean + u0 + v0, mean + u1 + v0, mean + u0 + v1, mean + u1 + v1};
    }
    V2 uv(V3 p) const {
        V3 d = p - mean;
        float lu = dot(d, axis_u), lv = dot(d, axis_v);
        V2 r;
        r.x = max_u > min_u + 1e-8f ? (lu - min_u) / (max_u - min_u) : 0.5f;
        r.y = max_v > min_v + 1e-8f ? (lv - min_v) / (max_v - min_v) : 0.5f;
        return r;
    }
    V3 longer_axis() const { return width_u() >= width_v() ? axis_u : axis_v; }
};

// src/bake.rs:794-826
void tight_bounds(const std::vector<V3>& pts, V3 mean, V3 au, V3 av, Frame& f) {
    if (pts.empty()) {
        f.min_u = -1e-3f; f.max_u = 1e-3f; f.min_v = -1e-3f; f.max_v = 1e-3f;
        return;
    }
    float mnu = 3.4e38f, mxu = -3.4e38f, mnv = 3.4e38f, mxv = -3.4e38f;
    for (auto& p : pts) {
        V3 d = p - mean;
        mnu = std::min(mnu, dot(d, au));
        mxu = std::max(mxu, dot(d, au));
        mnv = std::min(mnv, dot(d, av));
        mxv = std::max(mxv, dot(d, av));
    }
    float pad_u = std::max(mxu - mnu, 1e-3f) * 1e-3f + 1e-4f;
    float pad_v = std::max(mxv - mnv, 1e-3f) * 1e-3f + 1e-4f;
    mnu -= pad_u; mxu += pad_u; mnv -= pad_v; mxv += pad_v;
    if (mxu - mnu < 1e-2f) { float mid = (mxu + mnu) * 0.5f; mnu = mid - 5e-3f; mxu = mid + 5e-3f; }
    if (mxv - mnv < 1e-2f) { float mid = (mxv + mnv) * 0.5f; mnv = mid - 5e-3f; mxv = mid + 5e-3f; }
    f.min_u = mnu; f.max_u = mxu; f.min_v = mnv; f.max_v = mxv;
}

// src/bake.rs:716-732
Frame root_frame(const std::vector<Samples>& s) {
    std::vector<V3> pts;
    pts.reserve(s.size());
    for (auto& x : s) pts.push_back(x[0]);
    Frame f;
    V3 au, av;
    plane_axes(pts, f.mean, au, av);
    au = normalize_or(au, kX);
    av = normalize_or(av - au * dot(av, au), normalize_or(cross(au, kY), kZ));
    f.axis_u = au;
    f.axis_v = av;
    tight_bounds(pts, f.mean, au, av, f);
    return f;
}

// src/bake.rs:768-792
void transported_axes(V3 pu, V3 pv, V3 n, V3& au, V3& av) {
    V3 up = pu - n * dot(pu, n), vp = pv - n * dot(pv, n);
    float ul = len2(up), vl = len2(vp);
    if (ul >= vl && ul > 1e-8f) {
        au = up * (1.0f / len(up));
        av = cross(n, au);
        if (dot(av, pv) < 0.0f) av = -av;
        av = normalize_or(av, kX);
    } else if (vl > 1e-8f) {
        av = vp * (1.0f / len(vp));
        au = cross(av, n);
        if (dot(au, pu) < 0.0f) au = -au;
        au = normalize_or(au, kX);
    } else {
        au = normalize_or(cross(n, kY), kX);
        av = normalize_or(cross(n, au), kZ);
    }
}

// src/bake.rs:734-755
Frame oriented_frame(const std::vector<Samples>& s, size_t layer, V3 ru, V3 rv) {
    std::vector<V3> pts;
    pts.reserve(s.size());
    V3 tangent;
    for (auto& x : s) {
        pts.push_back(x[layer]);
        tangent += x[std::min(layer + 1, kLayers - 1)] - x[layer > 0 ? layer - 1 : 0];
    }
    Frame f;
    f.mean = average(pts);
    V3 n = normalize_or(tangent, kY);
    transported_axes(ru, rv, n, f.axis_u, f.axis_v);
    tight_bounds(pts, f.mean, f.axis_u, f.axis_v, f);
    return f;
}

// src/bake.rs:757-766
std::vector<Frame> frames_for(const std::vector<Samples>& s) {
    std::vector<Frame> fr;
    fr.reserve(kLayers);
    fr.push_back(root_frame(s));
    for (size_t l = 1; l < kLayers; ++l) fr.push_back(oriented_frame(s, l, fr[l - 1].axis_u, fr[l - 1].axis_v));
    return fr;
}

inline bool uv_in_unit(V2 uv) { return uv.x >= -1e-3f && uv.y >= -1e-3f && uv.x <= 1.0f + 1e-3f && uv.y <= 1.0f + 1e-3f; }

bool samples_inside(const std::vector<Frame>& fr, const Samples& s) {
    for (size_t l = 0; l < kLayers; ++l)
        if (!uv_in_unit(fr[l].uv(s[l]))) return false;
    return true;
}

inline V3 bilinear(const std::array<V3, 4>& q, V2 uv) {
    return q[0] * ((1 - uv.x) * (1 - uv.y)) + q[1] * (uv.x * (1 - uv.y)) + q[2] * ((1 - uv.x) * uv.y) + q[3] * (uv.x * uv.y);
}

// src/bake.rs:683-714
bool resample(const Strands& h, uint32_t strand, Samples& out) {
    auto [start, count] = h.strands[strand];
    if (count < 2) return false;
    const V3* pts = h.points + start;
    std::vector<float> cum(count, 0.0f);
    for (uint32_t i = 1; i < count; ++i) cum[i] = cum[i - 1] + dist(pts[i], pts[i - 1]);
    float length = cum[count - 1];
    if (length < 1e-5f) return false;
    for (size_t l = 0; l < kLayers; ++l) {
        float target = length * (float)l / (float)(kLayers - 1);
        uint32_t idx = 1;
        while (idx + 1 < count && cum[idx] < target) ++idx;
        float span = std::max(cum[idx] - cum[idx - 1], 1e-6f);
        float t = std::clamp((target - cum[idx - 1]) / span, 0.0f, 1.0f);
        out[l] = lerp(pts[idx - 1], pts[idx], t);
    }
    return true;
}

struct Indexed {
    std::vector<uint32_t> ids;
    std::vector<Samples> samples;
};

Indexed resample_indexed(const Strands& h, const std::vector<uint32_t>& group) {
    Indexed r;
    Samples s;
    for (uint32_t id : group) {
        if (resample(h, id, s)) {
            r.ids.push_back(id);
            r.samples.push_back(s);
        }
    }
    return r;
}

// src/bake.rs:1099-1123
void splat(std::vector<V3>& sum, std::vector<float>& weight, std::vector<float>* sum_sq, V2 uv, size_t layer, V3 res) {
    float u = std::clamp(uv.x, 0.0f, 1.0f) * (kStyleU - 1), v = std::clamp(uv.y, 0.0f, 1.0f) * (kStyleV - 1);
    uint32_t u0 = (uint32_t)std::floor(u), v0 = (uint32_t)std::floor(v);
    uint32_t u1 = std::min(u0 + 1, kStyleU - 1), v1 = std::min(v0 + 1, kStyleV - 1);
    float tu = u - u0, tv = v - v0;
    struct C { uint32_t iu, iv; float a; } cs[4] = {
        {u0, v0, (1 - tu) * (1 - tv)}, {u1, v0, tu * (1 - tv)}, {u0, v1, (1 - tu) * tv}, {u1, v1, tu * tv}};
    float l2 = len2(res);
    for (auto& c : cs) {
        if (c.a <= 0.0f) continue;
        size_t i = ((uint32_t)layer * kStyleV + c.iv) * kStyleU + c.iu;
        sum[i] += res * c.a;
        weight[i] += c.a;
        if (sum_sq) (*sum_sq)[i] += l2 * c.a;
    }
}

struct StyleFit {
    std::vector<V3> sum;
    std::vector<float> sum_sq, weight;
};

// src/bake.rs:845-889
StyleFit accumulate_style(const std::vector<Samples>& s, const std::vector<Frame>& fr) {
    StyleFit fit{std::vector<V3>(kStyleTexels), std::vector<float>(kStyleTexels, 0.0f),
                 std::vector<float>(kStyleTexels, 0.0f)};
    std::vector<std::array<V3, 4>> quads(kLayers);
    for (size_t l = 0; l < kLayers; ++l) quads[l] = fr[l].quad();
    for (auto& st : s) {
        V2 uv = fr[0].uv(st[0]);
        if (!uv_in_unit(uv)) continue;
        uv = clamp01(uv);
        for (size_t l = 0; l < kLayers; ++l) splat(fit.sum, fit.weight, &fit.sum_sq, uv, l, st[l] - bilinear(quads[l], uv));
    }
    return fit;
}

std::vector<V3> style_means(const StyleFit& fit) {
    std::vector<V3> st(kStyleTexels);
    for (size_t i = 0; i < kStyleTexels; ++i)
        if (fit.weight[i] > 0.0f) st[i] = fit.sum[i] / fit.weight[i];
    return st;
}

// src/bake.rs:906-923
std::pair<float, size_t> worst_stddev(const StyleFit& fit) {
    float worst = 0.0f;
    size_t layer = 0;
    for (size_t i = 0; i < kStyleTexels; ++i) {
        float w = fit.weight[i];
        if (w <= 1.0f) continue;
        V3 mean = fit.sum[i] / w;
        float second = fit.sum_sq[i] / w;
        float sd = std::sqrt(std::max(second - len2(mean), 0.0f));
        if (sd > worst) {
            worst = sd;
            layer = i / (kStyleU * kStyleV);
        }
    }
    return {worst, layer};
}

// src/bake.rs:925-943
V3 style_slice(const std::vector<V3>& st, V2 uv, size_t layer) {
    float u = std::clamp(uv.x, 0.0f, 1.0f) * (kStyleU - 1), v = std::clamp(uv.y, 0.0f, 1.0f) * (kStyleV - 1);
    uint32_t u0 = (uint32_t)std::floor(u), v0 = (uint32_t)std::floor(v);
    uint32_t u1 = std::min(u0 + 1, kStyleU - 1), v1 = std::min(v0 + 1, kStyleV - 1);
    float tu = u - u0, tv = v - v0;
    auto at = [&](uint32_t iu, uint32_t iv) { return st[((uint32_t)layer * kStyleV + iv) * kStyleU + iu]; };
    return lerp(lerp(at(u0, v0), at(u1, v0), tu), lerp(at(u0, v1), at(u1, v1), tu), tv);
}

// src/bake.rs:945-975
std::tuple<size_t, V3, float> worst_quad_gap(const std::vector<Samples>& s, const std::vector<Frame>& fr,
                                             const std::vector<V3>& st) {
    size_t worst_layer = 0;
    V3 worst_axis = fr[0].longer_axis();
    float worst = 0.0f;
    static const float ts[5] = {0.0f, 0.25f, 0.5f, 0.75f, 1.0f};
    for (size_t l = 0; l < kLayers; ++l) {
        auto quad = fr[l].quad();
        float gap = 0.0f;
        for (float v : ts) {
            for (float u : ts) {
                V2 uv{u, v};
                V3 pos = bilinear(quad, uv) + style_slice(st, uv, l);
                float nearest = 3.4e38f;
                for (auto& x : s) nearest = std::min(nearest, len2(pos - x[l]));
                gap = std::max(gap, nearest);
            }
        }
        gap = std::sqrt(gap);
        if (gap > worst) {
            worst = gap;
            worst_layer = l;
            worst_axis = fr[l].longer_axis();
        }
    }
    return {worst_layer, worst_axis, worst};
}

// src/bake.rs:1063-1088
std::tuple<float, size_t, V3> max_member_error(const std::vector<Samples>& s, const std::vector<Frame>& fr,
                                               const std::vector<V3>& st) {
    float worst = 0.0f;
    size_t layer = 0;
    V3 axis = fr[0].longer_axis();
    std::vector<std::array<V3, 4>> quads(kLayers);
    for (size_t l = 0; l < kLayers; ++l) quads[l] = fr[l].quad();
    for (auto& x : s) {
        V2 uv = fr[0].uv(x[0]);
        if (!uv_in_unit(uv)) continue;
        uv = clamp01(uv);
        for (size_t l = 0; l < kLayers; ++l) {
            float e = dist(bilinear(quads[l], uv) + style_slice(st, uv, l), x[l]);
            if (e > worst) {
                worst = e;
                layer = l;
                axis = fr[l].longer_axis();
            }
        }
    }
    return {worst, layer, axis};
}

// src/bake.rs:977-1061
void split_rec(const Strands& h, const std::vector<uint32_t>& group, uint32_t depth,
               std::vector<std::vector<uint32_t>>& out) {
    if (group.size() < 2 || depth >= 16) {
        out.push_back(group);
        return;
    }
    Indexed ix = resample_indexed(h, group);
    if (ix.ids.size() < 2) {
        out.push_back(ix.ids);
        return;
    }
    auto fr = frames_for(ix.samples);
    std::vector<uint32_t> inside, outside;
    for (size_t i = 0; i < ix.ids.size(); ++i)
        (samples_inside(fr, ix.samples[i]) ? inside : outside).push_back(ix.ids[i]);
    if (!outside.empty() && !inside.empty()) {
        split_rec(h, inside, depth + 1, out);
        split_rec(h, outside, depth + 1, out);
        return;
    }
    StyleFit fit = accumulate_style(ix.samples, fr);
    auto st = style_means(fit);
    auto [gap_layer, gap_axis, gap] = worst_quad_gap(ix.samples, fr, st);
    auto [stddev, var_layer] = worst_stddev(fit);
    auto [member_error, member_layer, member_axis] = max_member_error(ix.samples, fr, st);
    bool gap_bad = gap > kMaxQuadGap, var_bad = stddev > kMaxStyleStddev, member_bad = member_error > kMaxMemberError;
    if (!gap_bad && !var_bad && !member_bad) {
        out.push_back(ix.ids);
        return;
    }
    size_t layer;
    V3 axis;
    if (member_bad && member_error / kMaxMemberError >= gap / kMaxQuadGap &&
        member_error / kMaxMemberError >= stddev / std::max(kMaxStyleStddev, 1e-3f)) {
        layer = member_layer;
        axis = member_axis;
    } else if (var_bad && (!gap_bad || stddev / kMaxStyleStddev > gap / kMaxQuadGap)) {
        layer = std::min(var_layer, fr.size() - 1);
        axis = fr[layer].longer_axis();
    } else {
        layer = gap_layer;
        axis = gap_axis;
    }
    std::vector<V3> at_layer;
    for (auto& x : ix.samples) at_layer.push_back(x[layer]);
    V3 mean = average(at_layer);
    std::vector<std::pair<float, uint32_t>> order;
    for (size_t i = 0; i < ix.ids.size(); ++i) order.push_back({dot(ix.samples[i][layer] - mean, axis), ix.ids[i]});
    std::stable_sort(order.begin(), order.end(), [](auto& a, auto& b) { return a.first < b.first; });
    float span = order.back().first - order.front().first;
    size_t mid = order.size() / 2;
    if (mid == 0) {
        out.push_back(group);
        return;
    }
    std::vector<uint32_t> left, right;
    if (span < 1e-3f) {
        left.assign(group.begin(), group.begin() + mid);
        right.assign(group.begin() + mid, group.end());
    } else {
        for (size_t i = 0; i < order.size(); ++i) (i < mid ? left : right).push_back(order[i].second);
    }
    split_rec(h, left, depth + 1, out);
    split_rec(h, right, depth + 1, out);
}

// src/bake.rs:381-397
std::vector<std::vector<uint32_t>> split_along_axis(const std::vector<V3>& roots, const std::vector<uint32_t>& g) {
    std::vector<V3> pts;
    for (auto i : g) pts.push_back(roots[i]);
    V3 mean, axis, unused;
    plane_axes(pts, mean, axis, unused);
    std::vector<std::pair<float, uint32_t>> order;
    for (auto i : g) order.push_back({dot(roots[i] - mean, axis), i});
    std::stable_sort(order.begin(), order.end(), [](auto& a, auto& b) { return a.first < b.first; });
    if (order.back().first - order.front().first < 1e-3f) return {g};
    std::vector<std::vector<uint32_t>> out;
    size_t chunk = (size_t)kTargetStrandsPerCell;
    for (size_t i = 0; i < order.size(); i += chunk) {
        std::vector<uint32_t> piece;
        for (size_t j = i; j < std::min(order.size(), i + chunk); ++j) piece.push_back(order[j].second);
        out.push_back(piece);
    }
    return out;
}

// src/bake.rs:340-379
std::vector<std::vector<uint32_t>> cluster_roots_3d(const std::vector<V3>& roots, const std::vector<uint32_t>& which) {
    if (which.empty()) return {};
    if (which.size() <= (size_t)kTargetStrandsPerCell) return {which};
    V3 mn(3.4e38f, 3.4e38f, 3.4e38f), mx(-3.4e38f, -3.4e38f, -3.4e38f);
    for (auto i : which) { mn = vmin(mn, roots[i]); mx = vmax(mx, roots[i]); }
    V3 extent = vmax(mx - mn, V3(1e-3f, 1e-3f, 1e-3f));
    int cells = (int)std::clamp(std::ceil(std::cbrt((float)which.size() / kTargetStrandsPerCell)), 2.0f, 32.0f);
    V3 cell = extent / (float)cells;
    std::map<std::tuple<int, int, int>, std::vector<uint32_t>> buckets;
    for (auto i : which) {
        V3 p = roots[i] - mn;
        int kx = std::clamp((int)(p.x / cell.x), 0, cells - 1);
        int ky = std::clamp((int)(p.y / cell.y), 0, cells - 1);
        int kz = std::clamp((int)(p.z / cell.z), 0, cells - 1);
        buckets[{kx, ky, kz}].push_back(i);
    }
    std::vector<std::vector<uint32_t>> groups;
    for (auto& [key, g] : buckets) {
        if (g.size() > (size_t)kTargetStrandsPerCell * 2) {
            auto parts = split_along_axis(roots, g);
            groups.insert(groups.end(), parts.begin(), parts.end());
        } else {
            groups.push_back(g);
        }
    }
    return groups;
}

V3 centroid(const std::vector<uint32_t>& g, const std::vector<V3>& roots) {
    V3 acc;
    for (auto i : g) acc += roots[i];
    return acc / (float)std::max<size_t>(g.size(), 1);
}

// src/bake.rs:399-440
std::vector<std::vector<uint32_t>> absorb_sparse(std::vector<std::vector<uint32_t>> groups, const std::vector<V3>& roots) {
    groups.erase(std::remove_if(groups.begin(), groups.end(), [](auto& g) { return g.empty(); }), groups.end());
    if (groups.size() <= 1) return groups;
    std::vector<V3> cent;
    for (auto& g : groups) cent.push_back(centroid(g, roots));
    std::vector<bool> alive(groups.size(), true);
    float merge = kMaxQuadGap * kMaxQuadGap;
    for (size_t i = 0; i < groups.size(); ++i) {
        if (!alive[i] || groups[i].size() >= kMinStrandsPerBundle) continue;
        long best = -1;
        float best_d = 3.4e38f;
        for (size_t j = 0; j < groups.size(); ++j) {
            if (i == j || !alive[j]) continue;
            float d = len2(cent[i] - cent[j]);
            if (d < best_d) { best_d = d; best = (long)j; }
        }
        if (best < 0 || best_d > merge) continue;
        groups[best].insert(groups[best].end(), groups[i].begin(), groups[i].end());
        groups[i].clear();
        cent[best] = centroid(groups[best], roots);
        alive[i] = false;
    }
    std::vector<std::vector<uint32_t>> out;
    for (size_t i = 0; i < groups.size(); ++i)
        if (alive[i] && !groups[i].empty()) out.push_back(std::move(groups[i]));
    return out;
}

// ------------------------------------------------------------- ambient occlusion

struct KeyHash {
    size_t operator()(const std::tuple<int, int, int>& k) const {
        uint64_t h = (uint64_t)(uint32_t)std::get<0>(k) * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)(uint32_t)std::get<1>(k) * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)std::get<2>(k) * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

// src/bake.rs:1125-1282 (segments only: no scalp triangles here)
struct OccluderGrid {
    V3 origin;
    float cell = 4.0f;
    std::vector<std::pair<V3, V3>> segments;
    std::unordered_map<std::tuple<int, int, int>, std::vector<uint32_t>, KeyHash> buckets;

    std::tuple<int, int, int> key(V3 p) const {
        V3 q = (p - origin) / cell;
        return {(int)std::floor(q.x), (int)std::floor(q.y), (int)std::floor(q.z)};
    }

    explicit OccluderGrid(const Strands& h) {
        V3 mn(3.4e38f, 3.4e38f, 3.4e38f), mx(-3.4e38f, -3.4e38f, -3.4e38f);
        for (auto [start, count] : h.strands) {
            if (count < 2) continue;
            const V3* pts = h.points + start;
            size_t n = count;
            size_t step = (size_t)std::max(std::ceil((float)(n - 1) / 16.0f), 1.0f);
            size_t index = 0;
            while (index + 1 < n) {
                size_t next = std::min(index + step, n - 1);
                if (next > index) {
                    mn = vmin(vmin(mn, pts[index]), pts[next]);
                    mx = vmax(vmax(mx, pts[index]), pts[next]);
                    segments.push_back({pts[index], pts[next]});
                }
                if (next + 1 >= n) break;
                index = next;
            }
        }
        if (!std::isfinite(mn.x)) mn = V3();
        origin = mn;
        for (uint32_t i = 0; i < segments.size(); ++i) {
            auto [a, b] = segments[i];
            for (V3 p : {a, b, (a + b) * 0.5f}) buckets[key(p)].push_back(i);
        }
    }

    static bool ray_segment(V3 o, V3 d, V3 a, V3 b) {
        V3 ab = b - a, v = o - a;
        float d2 = dot(d, ab), d3 = std::max(len2(ab), 1e-12f), d4 = dot(v, d), d5 = dot(v, ab);
        float denom = d3 - d2 * d2;
        float s = std::fabs(denom) < 1e-8f ? 0.0f : std::clamp((d5 - d4 * d2) / denom, 0.0f, 1.0f);
        float t = dot(a + ab * s - o, d);
        if (!(t >= kAoMinT && t <= kAoReach)) {
            t = std::clamp(t, kAoMinT, kAoReach);
            s = std::clamp(dot(o + d * t - a, ab) / d3, 0.0f, 1.0f);
            t = dot(a + ab * s - o, d);
            if (!(t >= kAoMinT && t <= kAoReach)) return false;
        }
        return len2((o + d * t) - (a + ab * s)) <= kAoRadius * kAoRadius;
    }

    bool occluded(V3 o, V3 d) const {
        int steps = std::clamp((int)std::ceil(kAoReach / (cell * 0.5f)), 1, 8);
        float dt = kAoReach / (float)steps;
        for (int s = 0; s <= steps; ++s) {
            auto it = buckets.find(key(o + d * ((float)s * dt)));
            if (it == buckets.end()) continue;
            for (uint32_t i : it->second)
                if (ray_segment(o, d, segments[i].first, segments[i].second)) return true;
        }
        return false;
    }
};

// src/bake.rs:1284-1292
V3 hemisphere_dir(int index, int count, V3 normal) {
    float z = std::sqrt(((float)index + 0.5f) / (float)count);
    float phi = (float)index * 2.3999631f;
    float r = std::sqrt(std::max(1.0f - z * z, 0.0f));
    V3 local(r * std::cos(phi), r * std::sin(phi), z);
    V3 t = normalize_or(cross(normal, kY), kX);
    V3 b = normalize_or(cross(normal, t), kZ);
    return normalize_or(t * local.x + b * local.y + normal * local.z, normal);
}

}  // namespace

struct hg_bake_result {
    std::vector<hg_gpu_bundle> bundles;
    std::vector<hg_gpu_layer> layers;
    std::vector<float> style;
    float bounds[6];
};

extern "C" hg_bake_result* hg_bake(const float* points, uint32_t n_points, const uint32_t* first,
                                   const uint32_t* count, uint32_t n_strands, uint32_t flags) {
    if (!points || !first || !count) return nullptr;
    Strands h{reinterpret_cast<const V3*>(points), n_points, {}};
    h.strands.reserve(n_strands);
    for (uint32_t i = 0; i < n_strands; ++i) {
        if ((uint64_t)first[i] + count[i] > n_points) return nullptr;
        h.strands.push_back({first[i], count[i]});
    }
    auto* r = new (std::nothrow) hg_bake_result();
    if (!r) return nullptr;
    std::fill(r->bounds, r->bounds + 6, 0.0f);
    if (n_strands == 0) return r;

    std::vector<V3> roots(n_strands);
    std::vector<uint32_t> all(n_strands);
    for (uint32_t i = 0; i < n_strands; ++i) {
        roots[i] = h.points[first[i]];
        all[i] = i;
    }
    auto groups = absorb_sparse(cluster_roots_3d(roots, all), roots);

    // split_until_coherent per cluster, in parallel, kept in cluster order
    std::vector<std::vector<std::vector<uint32_t>>> split(groups.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (long g = 0; g < (long)groups.size(); ++g)
        if (!groups[g].empty()) split_rec(h, groups[g], 0, split[g]);
    std::vector<std::vector<uint32_t>> coherent;
    for (auto& s : split)
        for (auto& g : s) coherent.push_back(std::move(g));

    struct Built {
        bool ok = false;
        std::array<std::array<V3, 4>, kLayers> quads;
        std::vector<V3> style;
        uint32_t kept = 0;
    };
    std::vector<Built> built(coherent.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (long gi = 0; gi < (long)coherent.size(); ++gi) {
        Indexed ix = resample_indexed(h, coherent[gi]);
        if (ix.ids.empty()) continue;
        auto fr = frames_for(ix.samples);
        std::vector<Samples> kept;
        for (auto& s : ix.samples)
            if (samples_inside(fr, s)) kept.push_back(s);
        if (kept.empty()) continue;
        Built& b = built[gi];
        for (size_t l = 0; l < kLayers; ++l) b.quads[l] = fr[l].quad();
        std::vector<V3> sum(kStyleTexels);
        std::vector<float> weight(kStyleTexels, 0.0f);
        for (auto& s : kept) {
            V2 uv = fr[0].uv(s[0]);
            if (!uv_in_unit(uv)) continue;
            uv = clamp01(uv);
            for (size_t l = 0; l < kLayers; ++l)
                splat(sum, weight, nullptr, uv, l, s[l] - bilinear(b.quads[l], uv));
        }
        b.style.resize(kStyleTexels);
        for (size_t i = 0; i < kStyleTexels; ++i) b.style[i] = weight[i] > 0.0f ? sum[i] / weight[i] : V3();
        b.kept = (uint32_t)kept.size();
        b.ok = true;
    }

    V3 bmin(3.4e38f, 3.4e38f, 3.4e38f), bmax(-3.4e38f, -3.4e38f, -3.4e38f);
    std::vector<float> ao_tmp;
    for (auto& b : built) {
        if (!b.ok) continue;
        hg_gpu_bundle desc{(uint32_t)r->layers.size(), (uint32_t)(r->style.size() / 4), b.kept, 0u};
        for (size_t l = 0; l < kLayers; ++l) {
            for (int c = 0; c < 4; ++c) {
                bmin = vmin(bmin, b.quads[l][c]);
                bmax = vmax(bmax, b.quads[l][c]);
            }
        }
        // src/bake.rs:164-182
        for (size_t l = 0; l < kLayers; ++l) {
            auto& q = b.quads[l];
            auto& prev = b.quads[l > 0 ? l - 1 : 0];
            auto& next = b.quads[std::min(l + 1, kLayers - 1)];
            for (int c = 0; c < 4; ++c) {
                V3 t = l == 0 ? next[c] - q[c] : (l + 1 == kLayers ? q[c] - prev[c] : (next[c] - prev[c]) * 0.5f);
                hg_gpu_layer gl{{q[c].x, q[c].y, q[c].z, 1.0f}, {t.x, t.y, t.z, 0.0f}};
                r->layers.push_back(gl);
            }
        }
        for (auto& s : b.style) {
            r->style.push_back(s.x);
            r->style.push_back(s.y);
            r->style.push_back(s.z);
            r->style.push_back(0.0f);
        }
        r->bundles.push_back(desc);
    }
    if (r->bundles.empty()) return r;
    r->bounds[0] = bmin.x; r->bounds[1] = bmin.y; r->bounds[2] = bmin.z;
    r->bounds[3] = bmax.x; r->bounds[4] = bmax.y; r->bounds[5] = bmax.z;

    if (flags & HG_BAKE_AMBIENT_OCCLUSION) {
        // src/bake.rs:1139-1179
        OccluderGrid grid(h);
        std::vector<float> ao(r->layers.size(), 1.0f);
#pragma omp parallel for schedule(dynamic, 4)
        for (long bi = 0; bi < (long)r->bundles.size(); ++bi) {
            size_t base = r->bundles[bi].layer_offset;
            for (size_t l = 0; l < kLayers; ++l) {
                V3 center;
                for (int c = 0; c < 4; ++c) {
                    auto& p = r->layers[base + l * 4 + c].pos_ao;
                    center += V3(p[0], p[1], p[2]);
                }
                center = center * 0.25f;
                for (int c = 0; c < 4; ++c) {
                    size_t idx = base + l * 4 + c;
                    auto& gl = r->layers[idx];
                    V3 pos(gl.pos_ao[0], gl.pos_ao[1], gl.pos_ao[2]);
                    V3 tan = normalize_or(V3(gl.tangent[0], gl.tangent[1], gl.tangent[2]), kY);
                    V3 out = pos - center;
                    out -= tan * dot(out, tan);
                    out = normalize_or(out, normalize_or(cross(tan, kY), kX));
                    float occ = 0.0f;
                    for (int ray = 0; ray < kAoRays; ++ray)
                        if (grid.occluded(pos, hemisphere_dir(ray, kAoRays, out))) occ += 1.0f;
                    ao[idx] = std::clamp(1.0f - occ / (float)kAoRays, 0.0f, 1.0f);
                }
            }
        }
        for (size_t i = 0; i < ao.size(); ++i) r->layers[i].pos_ao[3] = ao[i];
    }
    return r;
}

extern "C" uint32_t hg_bake_bundle_count(const hg_bake_result* r) { return r ? (uint32_t)r->bundles.size() : 0u; }
extern "C" uint32_t hg_bake_layer_count(const hg_bake_result* r) { return r ? (uint32_t)r->layers.size() : 0u; }
extern "C" uint32_t hg_bake_style_count(const hg_bake_result* r) { return r ? (uint32_t)(r->style.size() / 4) : 0u; }

extern "C" void hg_bake_copy(const hg_bake_result* r, hg_gpu_bundle* bundles, hg_gpu_layer* layers, float* style,
                             float bounds[6]) {
    if (!r) return;
    if (bundles && !r->bundles.empty()) std::memcpy(bundles, r->bundles.data(), r->bundles.size() * sizeof(hg_gpu_bundle));
    if (layers && !r->layers.empty()) std::memcpy(layers, r->layers.data(), r->layers.size() * sizeof(hg_gpu_layer));
    if (style && !r->style.empty()) std::memcpy(style, r->style.data(), r->style.size() * sizeof(float));
    if (bounds) std::memcpy(bounds, r->bounds, sizeof(r->bounds));
}

extern "C" void hg_bake_free(hg_bake_result* r) { delete r; }
