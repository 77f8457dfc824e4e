// Hair-mesh baker: explicit strands (and optionally the scalp mesh they grow
// from) -> the bundle cages the per-frame pipeline generates strands from
// (GpuBundle / GpuLayer / style buffers, include/hairgb.h).  Host C++ with
// OpenMP; no counterpart of its algorithm in the reference, whose interface it
// replaces (bake_hair_mesh_with_scalp, src/bake.rs:89-213): the output only
// has to be valid bundles under the reference's own quality bounds (every
// strand in a bundle, roots inside their root quad, the uniform uv fill of
// each bundle close to the source strands, members reconstructed by the
// cage), which tests/test_baker.py checks.
//
// Pipeline:
//  1. every strand is resampled to 16 points at equal arc length;
//  2. strands are split top-down into bundles: a cluster that is too large
//     or not coherent is cut in two by 2-means on the whole resampled strands
//     (root points weighted up); with a scalp, clusters start per connected
//     scalp region of the roots' nearest triangles;
//  3. a cluster's cage: the root layer is a parallelogram spanned by the
//     principal axes of the roots in the plane across the strands (the scalp
//     normal there, when a scalp is given), which puts every root inside it
//     and fixes each member's (u, v); each further layer is the bilinear quad
//     that fits the members' points at their (u, v) best in the least-squares
//     sense (lightly pulled toward the root quad carried along the lock);
//  4. the style volume (8 x 8 texels per layer) is the regularised
//     least-squares fit of the members' remaining offsets, one Cholesky
//     factorisation per cluster;
//  5. a cluster is coherent when, evaluated exactly as the rasterizer
//     generates strands (bilinear layers, finite-difference tangents, Hermite
//     segments, trilinear style), every member is within kMemberError of its
//     resampled points, every root is within kRootPlane of the root quad's
//     plane, and a 5 x 5 uv grid at 31 heights stays within kGap of a member;
//  6. ambient occlusion per cage corner: Beer-Lambert transmittance
//     exp(-2 r * strand length per volume * path) along eight directions
//     across the lock, through a voxel grid of strand density (scalp cells
//     opaque), averaged.
// The bake is deterministic: parallel loops only read shared data and write
// per-item results, which are concatenated in a fixed order.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/hairgb_bake.h"

namespace {

constexpr int kLayers = HG_LAYER_COUNT;  // 16
constexpr int kSU = 8, kSV = 8, kSW = 16;
constexpr int kTexels = kSU * kSV;       // per layer
static_assert(kSW == kLayers, "one style layer per cage layer");

// Quality targets (asset units; the reference's tests bound the same
// quantities by 6 (reconstruction), 8 (stray) and 8 (root plane)).
constexpr float kMemberError = 3.5f;
constexpr float kGap = 4.5f;
constexpr float kRootPlane = 3.0f;
constexpr int kMaxMembers = 256;
constexpr float kMinWidth = 0.5f;        // smallest root-quad side
constexpr float kScalpAssign = 25.0f;    // roots farther from the scalp are clustered freely
constexpr float kAoRadius = 0.45f;       // fibre radius of the occlusion estimate
constexpr float kAoReach = 8.0f;
constexpr float kAoStart = 0.75f;

struct V3 {
    float x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float len(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 vmin(V3 a, V3 b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
inline V3 unit_or(V3 a, V3 fallback) {
    const float l = len(a);
    return l > 1e-12f && std::isfinite(l) ? a * (1.0f / l) : fallback;
}
// Any unit vector perpendicular to the unit vector d.
inline V3 perpendicular(V3 d) {
    const V3 t = std::fabs(d.x) < 0.8f ? V3{1.0f, 0.0f, 0.0f} : V3{0.0f, 1.0f, 0.0f};
    return unit_or(t - d * dot(t, d), {0.0f, 0.0f, 1.0f});
}
// The rotation by the smallest angle that takes unit a to unit b, applied to v.
inline V3 rotate_between(V3 a, V3 b, V3 v) {
    const V3 k = cross(a, b);
    const float c = dot(a, b), s = len(k);
    if (s < 1e-7f) return c > 0.0f ? v : v * -1.0f;
    const V3 axis = k * (1.0f / s);
    return v * c + cross(axis, v) * s + axis * (dot(axis, v) * (1.0f - c));
}

// Distance from p to segment ab.
inline float segment_distance(V3 p, V3 a, V3 b) {
    const V3 ab = b - a;
    const float d2 = dot(ab, ab);
    const float t = d2 > 1e-12f ? std::min(std::max(dot(p - a, ab) / d2, 0.0f), 1.0f) : 0.0f;
    return len(p - (a + ab * t));
}

// --------------------------------------------------------------- resampling

// 16 points at equal arc length along each strand with at least two points
// (a strand of zero length gives 16 copies of its root).
struct Resampled {
    std::vector<V3> pts;          // strand k: pts[k * 16 + layer]
    std::vector<uint32_t> source; // source strand index of strand k
    size_t count() const { return source.size(); }
    const V3* strand(size_t k) const { return &pts[k * kLayers]; }
};

Resampled resample(const float* points, const uint32_t* first, const uint32_t* count, uint32_t n) {
    Resampled r;
    for (uint32_t s = 0; s < n; ++s)
        if (count[s] >= 2) r.source.push_back(s);
    r.pts.resize(r.source.size() * kLayers);
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)r.source.size(); ++k) {
        const uint32_t s = r.source[(size_t)k];
        const float* p = points + 3u * first[s];
        const uint32_t m = count[s];
        auto at = [&](uint32_t i) { return V3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; };
        double total = 0.0;
        for (uint32_t i = 1; i < m; ++i) total += len(at(i) - at(i - 1));
        V3* out = &r.pts[(size_t)k * kLayers];
        uint32_t seg = 1;
        double walked = 0.0, seg_len = len(at(1) - at(0));
        for (int l = 0; l < kLayers; ++l) {
            const double goal = total * l / (kLayers - 1);
            while (seg + 1 < m && walked + seg_len < goal) {
                walked += seg_len;
                ++seg;
                seg_len = len(at(seg) - at(seg - 1));
            }
            const double t = seg_len > 1e-12 ? std::min(std::max((goal - walked) / seg_len, 0.0), 1.0) : 0.0;
            out[l] = at(seg - 1) + (at(seg) - at(seg - 1)) * (float)t;
        }
    }
    return r;
}

// --------------------------------------------------------------- scalp

struct Scalp {
    std::vector<V3> v;
    std::vector<uint32_t> tri;        // 3 per triangle
    std::vector<V3> normal;           // per triangle (winding as given)
    std::vector<uint32_t> component;  // connected region per triangle (shared vertices)
    // uniform grid of triangle bounding boxes
    V3 lo{0, 0, 0};
    float cell = 8.0f;
    int nx = 0, ny = 0, nz = 0;
    std::vector<uint32_t> start, items;
    size_t triangles() const { return tri.size() / 3; }
};

uint32_t find_root(std::vector<uint32_t>& parent, uint32_t a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
}

bool build_scalp(Scalp& sc, const float* verts, uint32_t n_verts, const uint32_t* idx, uint32_t n_idx) {
    sc.v.resize(n_verts);
    for (uint32_t i = 0; i < n_verts; ++i) sc.v[i] = {verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]};
    for (uint32_t i = 0; i + 2 < n_idx; i += 3) {
        if (idx[i] >= n_verts || idx[i + 1] >= n_verts || idx[i + 2] >= n_verts) return false;
        sc.tri.insert(sc.tri.end(), {idx[i], idx[i + 1], idx[i + 2]});
    }
    const size_t nt = sc.triangles();
    if (nt == 0) return true;
    sc.normal.resize(nt);
    std::vector<uint32_t> parent(n_verts);
    std::iota(parent.begin(), parent.end(), 0u);
    V3 lo{3e38f, 3e38f, 3e38f}, hi{-3e38f, -3e38f, -3e38f};
    for (size_t t = 0; t < nt; ++t) {
        const V3 a = sc.v[sc.tri[3 * t]], b = sc.v[sc.tri[3 * t + 1]], c = sc.v[sc.tri[3 * t + 2]];
        sc.normal[t] = unit_or(cross(b - a, c - a), {0.0f, 1.0f, 0.0f});
        lo = vmin(lo, vmin(a, vmin(b, c)));
        hi = vmax(hi, vmax(a, vmax(b, c)));
        const uint32_t r0 = find_root(parent, sc.tri[3 * t]);
        for (int k = 1; k < 3; ++k) {
            const uint32_t rk = find_root(parent, sc.tri[3 * t + k]);
            if (rk != r0) parent[rk] = r0;
        }
    }
    sc.component.resize(nt);
    for (size_t t = 0; t < nt; ++t) sc.component[t] = find_root(parent, sc.tri[3 * t]);
    sc.lo = lo;
    const V3 ext = hi - lo;
    sc.cell = std::max(8.0f, std::max(ext.x, std::max(ext.y, ext.z)) / 128.0f);
    sc.nx = std::max(1, (int)std::ceil(ext.x / sc.cell) + 1);
    sc.ny = std::max(1, (int)std::ceil(ext.y / sc.cell) + 1);
    sc.nz = std::max(1, (int)std::ceil(ext.z / sc.cell) + 1);
    const size_t cells = (size_t)sc.nx * sc.ny * sc.nz;
    std::vector<uint32_t> cnt(cells + 1, 0);
    auto cell_range = [&](size_t t, int r[6]) {
        const V3 a = sc.v[sc.tri[3 * t]], b = sc.v[sc.tri[3 * t + 1]], c = sc.v[sc.tri[3 * t + 2]];
        const V3 mn = vmin(a, vmin(b, c)) - lo, mx = vmax(a, vmax(b, c)) - lo;
        r[0] = std::min(sc.nx - 1, (int)(mn.x / sc.cell));
        r[1] = std::min(sc.ny - 1, (int)(mn.y / sc.cell));
        r[2] = std::min(sc.nz - 1, (int)(mn.z / sc.cell));
        r[3] = std::min(sc.nx - 1, (int)(mx.x / sc.cell));
        r[4] = std::min(sc.ny - 1, (int)(mx.y / sc.cell));
        r[5] = std::min(sc.nz - 1, (int)(mx.z / sc.cell));
    };
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            sc.start.assign(cells + 1, 0);
            for (size_t c = 0; c < cells; ++c) sc.start[c + 1] = sc.start[c] + cnt[c];
            sc.items.resize(sc.start[cells]);
            std::fill(cnt.begin(), cnt.end(), 0u);
        }
        for (size_t t = 0; t < nt; ++t) {
            int r[6];
            cell_range(t, r);
            for (int z = r[2]; z <= r[5]; ++z)
                for (int y = r[1]; y <= r[4]; ++y)
                    for (int x = r[0]; x <= r[3]; ++x) {
                        const size_t c = ((size_t)z * sc.ny + y) * sc.nx + x;
                        if (pass == 1) sc.items[sc.start[c] + cnt[c]] = (uint32_t)t;
                        ++cnt[c];
                    }
        }
    }
    return true;
}

// Closest point of triangle abc to p: the plane projection when it falls
// inside, else the closest of the three edges.
V3 closest_on_triangle(V3 p, V3 a, V3 b, V3 c) {
    const V3 n = cross(b - a, c - a);
    const float n2 = dot(n, n);
    if (n2 > 1e-20f) {
        const V3 q = p - n * (dot(p - a, n) / n2);
        const float wa = dot(cross(b - q, c - q), n), wb = dot(cross(c - q, a - q), n), wc = dot(cross(a - q, b - q), n);
        if (wa >= 0.0f && wb >= 0.0f && wc >= 0.0f) return q;
    }
    V3 best = a;
    float bd = 3e38f;
    const V3 e[3][2] = {{a, b}, {b, c}, {c, a}};
    for (const auto& s : e) {
        const V3 ab = s[1] - s[0];
        const float d2 = dot(ab, ab);
        const float t = d2 > 1e-20f ? std::min(std::max(dot(p - s[0], ab) / d2, 0.0f), 1.0f) : 0.0f;
        const V3 q = s[0] + ab * t;
        const float d = len(p - q);
        if (d < bd) {
            bd = d;
            best = q;
        }
    }
    return best;
}

// Nearest triangle within max_dist (-1 when none).
long long nearest_triangle(const Scalp& sc, V3 p, float max_dist, float* dist) {
    if (sc.triangles() == 0) return -1;
    const V3 q = p - sc.lo;
    const int cx = (int)std::floor(q.x / sc.cell), cy = (int)std::floor(q.y / sc.cell),
              cz = (int)std::floor(q.z / sc.cell);
    const int reach = (int)std::ceil(max_dist / sc.cell);
    long long best = -1;
    float bd = max_dist;
    for (int z = cz - reach; z <= cz + reach; ++z)
        for (int y = cy - reach; y <= cy + reach; ++y)
            for (int x = cx - reach; x <= cx + reach; ++x) {
                if (x < 0 || y < 0 || z < 0 || x >= sc.nx || y >= sc.ny || z >= sc.nz) continue;
                const size_t c = ((size_t)z * sc.ny + y) * sc.nx + x;
                for (uint32_t i = sc.start[c]; i < sc.start[c + 1]; ++i) {
                    const uint32_t t = sc.items[i];
                    const V3 cp = closest_on_triangle(p, sc.v[sc.tri[3 * t]], sc.v[sc.tri[3 * t + 1]],
                                                      sc.v[sc.tri[3 * t + 2]]);
                    const float d = len(p - cp);
                    if (d < bd || (d == bd && best >= 0 && (long long)t < best)) {
                        bd = d;
                        best = t;
                    }
                }
            }
    *dist = bd;
    return best;
}

// --------------------------------------------------------------- cages

struct Cage {
    V3 q[kLayers][4];                    // corners c00, c10, c01, c11 per layer
    std::array<V3, kLayers * kTexels> style;  // [layer][v][u]
};

// Bilinear weights of (u, v) for c00, c10, c01, c11 (the shader's order).
inline std::array<float, 4> bilinear_w(float u, float v) {
    return {(1.0f - u) * (1.0f - v), u * (1.0f - v), (1.0f - u) * v, u * v};
}
inline V3 bilinear(const V3 q[4], float u, float v) {
    const auto w = bilinear_w(u, v);
    return ((q[0] * w[0] + q[1] * w[1]) + q[2] * w[2]) + q[3] * w[3];
}

// Style texel weights of (u, v) within a layer: 4 texel indices and weights.
inline void style_w(float u, float v, int idx[4], float w[4]) {
    const float uu = std::min(std::max(u, 0.0f), 1.0f) * (kSU - 1), vv = std::min(std::max(v, 0.0f), 1.0f) * (kSV - 1);
    const int u0 = std::min((int)std::floor(uu), kSU - 1), v0 = std::min((int)std::floor(vv), kSV - 1);
    const int u1 = std::min(u0 + 1, kSU - 1), v1 = std::min(v0 + 1, kSV - 1);
    const float tu = uu - (float)u0, tv = vv - (float)v0;
    idx[0] = v0 * kSU + u0, w[0] = (1.0f - tu) * (1.0f - tv);
    idx[1] = v0 * kSU + u1, w[1] = tu * (1.0f - tv);
    idx[2] = v1 * kSU + u0, w[2] = (1.0f - tu) * tv;
    idx[3] = v1 * kSU + u1, w[3] = tu * tv;
}

inline V3 style_at(const Cage& c, int layer, float u, float v) {
    int idx[4];
    float w[4];
    style_w(u, v, idx, w);
    V3 r{0, 0, 0};
    for (int k = 0; k < 4; ++k) r = r + c.style[layer * kTexels + idx[k]] * w[k];
    return r;
}

// Strand position at (u, v, w) as the rasterizer generates it: bilinear
// layer points, finite-difference tangents of those, a Hermite segment
// between the two layers around w, and the trilinear style residual.
V3 generated_point(const Cage& c, float u, float v, float w) {
    const float lf = std::min(std::max(w, 0.0f), 1.0f) * (kLayers - 1);
    const int i0 = std::min((int)std::floor(lf), kLayers - 1), i1 = std::min(i0 + 1, kLayers - 1);
    const float t = lf - (float)i0;
    auto point = [&](int l) { return bilinear(c.q[std::min(std::max(l, 0), kLayers - 1)], u, v); };
    auto tangent = [&](int l) {
        V3 d;
        float s;
        if (l == 0) {
            d = point(1) - point(0);
            s = len(d);
        } else if (l == kLayers - 1) {
            d = point(l) - point(l - 1);
            s = len(d);
        } else {
            d = point(l + 1) - point(l - 1);
            s = 0.5f * len(d);
        }
        return unit_or(d, {0.0f, 1.0f, 0.0f}) * std::max(s, 1e-4f);
    };
    const V3 p0 = point(i0), p1 = point(i1), m0 = tangent(i0), m1 = tangent(i1);
    const float t2 = t * t, t3 = t2 * t;
    const V3 base = p0 * (2 * t3 - 3 * t2 + 1) + m0 * (t3 - 2 * t2 + t) + p1 * (-2 * t3 + 3 * t2) + m1 * (t3 - t2);
    // trilinear style: the two layers' bilinear residuals, lerped in w
    const float ww = std::min(std::max(w, 0.0f), 1.0f) * (kSW - 1);
    const int w0 = std::min((int)std::floor(ww), kSW - 1), w1 = std::min(w0 + 1, kSW - 1);
    const float tw = ww - (float)w0;
    const V3 s0 = style_at(c, w0, u, v), s1 = style_at(c, w1, u, v);
    return base + s0 + (s1 - s0) * tw;
}

// Symmetric positive definite solve by Cholesky (n <= 64), in place; false
// when the matrix is not positive definite.
template <int N>
bool cholesky(std::array<double, N * N>& a) {
    for (int j = 0; j < N; ++j) {
        double d = a[j * N + j];
        for (int k = 0; k < j; ++k) d -= a[j * N + k] * a[j * N + k];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        a[j * N + j] = d;
        for (int i = j + 1; i < N; ++i) {
            double s = a[i * N + j];
            for (int k = 0; k < j; ++k) s -= a[i * N + k] * a[j * N + k];
            a[i * N + j] = s / d;
        }
    }
    return true;
}
template <int N>
void cholesky_solve(const std::array<double, N * N>& l, double* x) {
    for (int i = 0; i < N; ++i) {
        double s = x[i];
        for (int k = 0; k < i; ++k) s -= l[i * N + k] * x[k];
        x[i] = s / l[i * N + i];
    }
    for (int i = N - 1; i >= 0; --i) {
        double s = x[i];
        for (int k = i + 1; k < N; ++k) s -= l[k * N + i] * x[k];
        x[i] = s / l[i * N + i];
    }
}

struct Fit {
    Cage cage;
    std::vector<float> u, v;  // members' root uv
    bool coherent = false;
};

struct Context {
    const Resampled* rs = nullptr;
    const Scalp* scalp = nullptr;
    std::vector<V3> root_normal;  // per resampled strand: scalp normal at its root, or zero
};

// Cage, style and coherence of the cluster `m` (indices into the resampled strands).
Fit fit_cluster(const Context& cx, const std::vector<uint32_t>& m) {
    const Resampled& rs = *cx.rs;
    const size_t n = m.size();
    Fit f;
    f.u.resize(n);
    f.v.resize(n);
    V3 centre[kLayers];
    for (int l = 0; l < kLayers; ++l) {
        double sx = 0, sy = 0, sz = 0;
        for (uint32_t k : m) {
            const V3 p = rs.strand(k)[l];
            sx += p.x, sy += p.y, sz += p.z;
        }
        centre[l] = {(float)(sx / n), (float)(sy / n), (float)(sz / n)};
    }
    // direction of the lock per layer
    V3 dir[kLayers];
    for (int l = 0; l < kLayers; ++l) {
        const V3 d = centre[std::min(l + 1, kLayers - 1)] - centre[std::max(l - 1, 0)];
        dir[l] = unit_or(d, l > 0 ? dir[l - 1] : V3{0.0f, 1.0f, 0.0f});
    }
    // root plane: across the strands, or along the scalp normal under them
    V3 d0 = dir[0];
    {
        V3 ns{0, 0, 0};
        for (uint32_t k : m) ns = ns + cx.root_normal[k];
        if (len(ns) > 1e-6f) {
            V3 sn = unit_or(ns, d0);
            if (dot(sn, dir[0]) < 0.0f) sn = sn * -1.0f;  // outward, along the hair
            d0 = sn;
        }
    }
    const V3 a = perpendicular(d0), b = cross(d0, a);
    double cxx = 0, cxy = 0, cyy = 0;
    for (uint32_t k : m) {
        const V3 r = rs.strand(k)[0] - centre[0];
        const double x = dot(r, a), y = dot(r, b);
        cxx += x * x, cxy += x * y, cyy += y * y;
    }
    const float theta = 0.5f * (float)std::atan2(2.0 * cxy, cxx - cyy);
    const V3 e1 = a * std::cos(theta) + b * std::sin(theta), e2 = cross(d0, e1);
    float s0 = 3e38f, s1 = -3e38f, t0 = 3e38f, t1 = -3e38f, plane = 0.0f;
    for (uint32_t k : m) {
        const V3 r = rs.strand(k)[0] - centre[0];
        const float s = dot(r, e1), t = dot(r, e2);
        s0 = std::min(s0, s), s1 = std::max(s1, s);
        t0 = std::min(t0, t), t1 = std::max(t1, t);
        plane = std::max(plane, std::fabs(dot(r, d0)));
    }
    auto widen = [](float& lo, float& hi) {
        const float w = hi - lo;
        const float pad = std::max(0.5f * (kMinWidth - w), 0.0f) + std::max(1e-3f, 1e-3f * w);
        lo -= pad, hi += pad;
    };
    widen(s0, s1);
    widen(t0, t1);
    Cage& c = f.cage;
    c.q[0][0] = centre[0] + e1 * s0 + e2 * t0;
    c.q[0][1] = centre[0] + e1 * s1 + e2 * t0;
    c.q[0][2] = centre[0] + e1 * s0 + e2 * t1;
    c.q[0][3] = centre[0] + e1 * s1 + e2 * t1;
    for (size_t i = 0; i < n; ++i) {
        const V3 r = rs.strand(m[i])[0] - centre[0];
        f.u[i] = (dot(r, e1) - s0) / (s1 - s0);
        f.v[i] = (dot(r, e2) - t0) / (t1 - t0);
    }
    // further layers: least-squares bilinear quads at the members' (u, v),
    // pulled lightly toward the root quad carried along the lock
    std::array<double, 16> nrm{};
    for (size_t i = 0; i < n; ++i) {
        const auto w = bilinear_w(f.u[i], f.v[i]);
        for (int r = 0; r < 4; ++r)
            for (int q = 0; q < 4; ++q) nrm[r * 4 + q] += (double)w[r] * w[q];
    }
    const double lambda = 1e-3 * (double)n + 1e-3;
    std::array<double, 16> chol = nrm;
    for (int r = 0; r < 4; ++r) chol[r * 4 + r] += lambda;
    cholesky<4>(chol);  // positive definite by the ridge
    for (int l = 1; l < kLayers; ++l) {
        double rhs[3][4] = {};
        for (size_t i = 0; i < n; ++i) {
            const auto w = bilinear_w(f.u[i], f.v[i]);
            const V3 p = rs.strand(m[i])[l];
            for (int r = 0; r < 4; ++r) rhs[0][r] += w[r] * p.x, rhs[1][r] += w[r] * p.y, rhs[2][r] += w[r] * p.z;
        }
        V3 prior[4];
        for (int r = 0; r < 4; ++r) prior[r] = centre[l] + rotate_between(d0, dir[l], c.q[0][r] - centre[0]);
        for (int r = 0; r < 4; ++r)
            rhs[0][r] += lambda * prior[r].x, rhs[1][r] += lambda * prior[r].y, rhs[2][r] += lambda * prior[r].z;
        for (int d = 0; d < 3; ++d) cholesky_solve<4>(chol, rhs[d]);
        for (int r = 0; r < 4; ++r) c.q[l][r] = {(float)rhs[0][r], (float)rhs[1][r], (float)rhs[2][r]};
    }
    // style: regularised least squares of the members' offsets from the
    // bilinear quads, the same 64 x 64 system for every layer and axis
    {
        std::array<double, kTexels * kTexels> A{};
        std::vector<std::array<int, 4>> ti(n);
        std::vector<std::array<float, 4>> tw(n);
        for (size_t i = 0; i < n; ++i) {
            style_w(f.u[i], f.v[i], ti[i].data(), tw[i].data());
            for (int r = 0; r < 4; ++r)
                for (int q = 0; q < 4; ++q) A[ti[i][r] * kTexels + ti[i][q]] += (double)tw[i][r] * tw[i][q];
        }
        // smoothness between neighbouring texels and a small ridge
        const double smooth = 0.02 * ((double)n / kTexels + 1.0), ridge = 1e-4;
        for (int vv = 0; vv < kSV; ++vv)
            for (int uu = 0; uu < kSU; ++uu) {
                const int i = vv * kSU + uu;
                A[i * kTexels + i] += ridge;
                const int nb[2] = {uu + 1 < kSU ? i + 1 : -1, vv + 1 < kSV ? i + kSU : -1};
                for (int j : nb) {
                    if (j < 0) continue;
                    A[i * kTexels + i] += smooth, A[j * kTexels + j] += smooth;
                    A[i * kTexels + j] -= smooth, A[j * kTexels + i] -= smooth;
                }
            }
        const bool ok = cholesky<kTexels>(A);
        for (int l = 0; l < kLayers; ++l) {
            double rhs[3][kTexels] = {};
            for (size_t i = 0; i < n; ++i) {
                const V3 res = rs.strand(m[i])[l] - bilinear(c.q[l], f.u[i], f.v[i]);
                for (int r = 0; r < 4; ++r) {
                    rhs[0][ti[i][r]] += tw[i][r] * res.x;
                    rhs[1][ti[i][r]] += tw[i][r] * res.y;
                    rhs[2][ti[i][r]] += tw[i][r] * res.z;
                }
            }
            if (ok)
                for (int d = 0; d < 3; ++d) cholesky_solve<kTexels>(A, rhs[d]);
            for (int t = 0; t < kTexels; ++t)
                c.style[l * kTexels + t] = ok ? V3{(float)rhs[0][t], (float)rhs[1][t], (float)rhs[2][t]} : V3{0, 0, 0};
        }
    }
    // coherence
    if (n > (size_t)kMaxMembers || plane > kRootPlane) return f;
    for (size_t i = 0; i < n; ++i)
        for (int l = 0; l < kLayers; ++l) {
            const V3 p = generated_point(c, f.u[i], f.v[i], (float)l / (kLayers - 1));
            if (len(p - rs.strand(m[i])[l]) > kMemberError) return f;
        }
    for (int step = 0; step < 2 * kLayers - 1; ++step) {
        const float w = (float)step / (2 * kLayers - 2);
        const int l = std::min(step / 2, kLayers - 2);
        for (int gv = 0; gv < 5; ++gv)
            for (int gu = 0; gu < 5; ++gu) {
                const V3 p = generated_point(c, 0.25f * gu, 0.25f * gv, w);
                float best = 3e38f;
                for (size_t i = 0; i < n && best > kGap; ++i) {
                    const V3* s = rs.strand(m[i]);
                    for (int j = std::max(l - 1, 0); j <= std::min(l + 1, kLayers - 2) && best > kGap; ++j)
                        best = std::min(best, segment_distance(p, s[j], s[j + 1]));
                }
                if (best > kGap) return f;
            }
    }
    f.coherent = true;
    return f;
}

// Two halves of a cluster by 2-means on the resampled strands (squared
// distances, root points weighted up), seeded with a far-apart pair.
void split_cluster(const Resampled& rs, const std::vector<uint32_t>& m, std::vector<uint32_t>& a,
                   std::vector<uint32_t>& b) {
    float wt[kLayers];
    for (int l = 0; l < kLayers; ++l) wt[l] = 1.0f + 2.0f * (float)(kLayers - 1 - l) / (kLayers - 1);
    auto dist2 = [&](const V3* x, const V3* y) {
        float s = 0.0f;
        for (int l = 0; l < kLayers; ++l) {
            const V3 d = x[l] - y[l];
            s += wt[l] * dot(d, d);
        }
        return s;
    };
    std::vector<V3> mean(kLayers, V3{0, 0, 0});
    for (uint32_t k : m)
        for (int l = 0; l < kLayers; ++l) mean[l] = mean[l] + rs.strand(k)[l] * (1.0f / (float)m.size());
    auto farthest = [&](const V3* from) {
        uint32_t best = m[0];
        float bd = -1.0f;
        for (uint32_t k : m) {
            const float d = dist2(rs.strand(k), from);
            if (d > bd) bd = d, best = k;
        }
        return best;
    };
    const uint32_t sa = farthest(mean.data()), sb = farthest(rs.strand(sa));
    std::vector<V3> ca(rs.strand(sa), rs.strand(sa) + kLayers), cb(rs.strand(sb), rs.strand(sb) + kLayers);
    std::vector<uint8_t> side(m.size(), 0);
    for (int it = 0; it < 12; ++it) {
        bool changed = false;
        std::vector<V3> na(kLayers, V3{0, 0, 0}), nb(kLayers, V3{0, 0, 0});
        size_t count_a = 0, count_b = 0;
        for (size_t i = 0; i < m.size(); ++i) {
            const V3* s = rs.strand(m[i]);
            const uint8_t sd = dist2(s, cb.data()) < dist2(s, ca.data()) ? 1 : 0;
            changed |= sd != side[i];
            side[i] = sd;
            auto& acc = sd ? nb : na;
            for (int l = 0; l < kLayers; ++l) acc[l] = acc[l] + s[l];
            (sd ? count_b : count_a) += 1;
        }
        if (count_a == 0 || count_b == 0) break;
        for (int l = 0; l < kLayers; ++l) ca[l] = na[l] * (1.0f / count_a), cb[l] = nb[l] * (1.0f / count_b);
        if (!changed && it > 0) break;
    }
    a.clear();
    b.clear();
    for (size_t i = 0; i < m.size(); ++i) (side[i] ? b : a).push_back(m[i]);
    if (a.empty() || b.empty()) {  // identical strands: halves in order
        a.assign(m.begin(), m.begin() + m.size() / 2);
        b.assign(m.begin() + m.size() / 2, m.end());
    }
}

// --------------------------------------------------------------- ambient occlusion

struct Density {
    V3 lo{0, 0, 0};
    float h = 1.0f;
    int nx = 1, ny = 1, nz = 1;
    std::vector<float> rho;      // strand length per cell volume
    std::vector<uint8_t> solid;  // scalp cells
    // Density trilinear between cell centres (so a strand's two ends read
    // alike wherever the cell boundaries fall); opaque from the cell itself.
    float at(V3 p, bool* opaque) const {
        const V3 q = (p - lo) * (1.0f / h);
        const int cx = (int)std::floor(q.x), cy = (int)std::floor(q.y), cz = (int)std::floor(q.z);
        if (cx >= 0 && cy >= 0 && cz >= 0 && cx < nx && cy < ny && cz < nz)
            *opaque = solid[((size_t)cz * ny + cy) * nx + cx] != 0;
        const float fx = q.x - 0.5f, fy = q.y - 0.5f, fz = q.z - 0.5f;
        const int x0 = (int)std::floor(fx), y0 = (int)std::floor(fy), z0 = (int)std::floor(fz);
        const float tx = fx - x0, ty = fy - y0, tz = fz - z0;
        float r = 0.0f;
        for (int k = 0; k < 8; ++k) {
            const int x = x0 + (k & 1), y = y0 + ((k >> 1) & 1), z = z0 + (k >> 2);
            if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
            const float w = ((k & 1) ? tx : 1.0f - tx) * (((k >> 1) & 1) ? ty : 1.0f - ty) * ((k >> 2) ? tz : 1.0f - tz);
            r += w * rho[((size_t)z * ny + y) * nx + x];
        }
        return r;
    }
};

Density build_density(const Resampled& rs, const Scalp* scalp) {
    Density g;
    V3 lo{3e38f, 3e38f, 3e38f}, hi{-3e38f, -3e38f, -3e38f};
    for (const V3& p : rs.pts) lo = vmin(lo, p), hi = vmax(hi, p);
    lo = lo - V3{kAoReach, kAoReach, kAoReach};
    hi = hi + V3{kAoReach, kAoReach, kAoReach};
    const V3 ext = hi - lo;
    g.h = std::max(1.0f, std::max(ext.x, std::max(ext.y, ext.z)) / 256.0f);
    g.lo = lo;
    g.nx = std::max(1, (int)std::ceil(ext.x / g.h));
    g.ny = std::max(1, (int)std::ceil(ext.y / g.h));
    g.nz = std::max(1, (int)std::ceil(ext.z / g.h));
    const size_t cells = (size_t)g.nx * g.ny * g.nz;
    g.rho.assign(cells, 0.0f);
    g.solid.assign(cells, 0);
    const float vol = g.h * g.h * g.h;
    auto cell_of = [&](V3 p, size_t* c) {
        const V3 q = (p - g.lo) * (1.0f / g.h);
        const int x = (int)std::floor(q.x), y = (int)std::floor(q.y), z = (int)std::floor(q.z);
        if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) return false;
        *c = ((size_t)z * g.ny + y) * g.nx + x;
        return true;
    };
    for (size_t k = 0; k < rs.count(); ++k) {
        const V3* s = rs.strand(k);
        for (int l = 0; l + 1 < kLayers; ++l) {
            const float sl = len(s[l + 1] - s[l]);
            const int steps = std::max(1, (int)std::ceil(2.0f * sl / g.h));
            for (int i = 0; i < steps; ++i) {
                size_t c;
                if (cell_of(s[l] + (s[l + 1] - s[l]) * ((i + 0.5f) / steps), &c)) g.rho[c] += sl / steps / vol;
            }
        }
    }
    if (scalp) {
        for (size_t t = 0; t < scalp->triangles(); ++t) {
            const V3 a = scalp->v[scalp->tri[3 * t]], b = scalp->v[scalp->tri[3 * t + 1]],
                     c = scalp->v[scalp->tri[3 * t + 2]];
            const float e = std::max(len(b - a), std::max(len(c - a), len(c - b)));
            const int steps = std::max(1, (int)std::ceil(2.0f * e / g.h));
            for (int i = 0; i <= steps; ++i)
                for (int j = 0; i + j <= steps; ++j) {
                    size_t cc;
                    if (cell_of(a + (b - a) * ((float)i / steps) + (c - a) * ((float)j / steps), &cc)) g.solid[cc] = 1;
                }
        }
    }
    return g;
}

// Transmittance averaged over eight directions across the local strand
// direction d: exp(-2 r * integral of strand density) from kAoStart to
// kAoReach, zero where a scalp cell is met.
float corner_ao(const Density& g, V3 p, V3 d) {
    const V3 a = perpendicular(d), b = cross(d, a);
    const float step = 0.5f * g.h;
    float sum = 0.0f;
    for (int k = 0; k < 8; ++k) {
        const float ang = 0.78539816f * k;
        const V3 dir = a * std::cos(ang) + b * std::sin(ang);
        float tau = 0.0f;
        bool blocked = false;
        for (float t = kAoStart; t < kAoReach && !blocked; t += step) {
            bool opaque = false;
            tau += g.at(p + dir * t, &opaque) * step;
            blocked = opaque;
        }
        sum += blocked ? 0.0f : std::exp(-2.0f * kAoRadius * tau);
    }
    return sum / 8.0f;
}

}  // namespace

struct hg_bake_result {
    std::vector<hg_gpu_bundle> bundles;
    std::vector<hg_gpu_layer> layers;
    std::vector<float> style;  // 4 per texel
    float bounds[6] = {0, 0, 0, 0, 0, 0};
};

namespace {

hg_bake_result* bake(const float* points, uint32_t n_points, const uint32_t* first, const uint32_t* count,
                     uint32_t n_strands, const float* scalp_v, uint32_t n_scalp_v, const uint32_t* scalp_i,
                     uint32_t n_scalp_i, uint32_t flags) {
    if (n_strands && (!points || !first || !count)) return nullptr;
    for (uint32_t s = 0; s < n_strands; ++s)
        if ((uint64_t)first[s] + count[s] > n_points) return nullptr;
    Scalp scalp;
    const bool has_scalp = scalp_v && scalp_i && n_scalp_v && n_scalp_i >= 3;
    if (has_scalp && !build_scalp(scalp, scalp_v, n_scalp_v, scalp_i, n_scalp_i)) return nullptr;
    hg_bake_result* out = new (std::nothrow) hg_bake_result();
    if (!out) return nullptr;
    const Resampled rs = resample(points, first, count, n_strands);
    if (rs.count() == 0) return out;
    Context cx;
    cx.rs = &rs;
    cx.scalp = has_scalp ? &scalp : nullptr;
    cx.root_normal.assign(rs.count(), V3{0, 0, 0});
    // initial clusters: one, or one per connected scalp region of the roots'
    // nearest triangles (roots far from the scalp form their own cluster)
    std::vector<std::vector<uint32_t>> work;
    if (has_scalp && scalp.triangles()) {
        std::vector<long long> region(rs.count(), -1);
#pragma omp parallel for schedule(dynamic, 256)
        for (long long k = 0; k < (long long)rs.count(); ++k) {
            float d = 0.0f;
            const long long t = nearest_triangle(scalp, rs.strand((size_t)k)[0], kScalpAssign, &d);
            if (t >= 0) {
                region[(size_t)k] = scalp.component[(size_t)t];
                cx.root_normal[(size_t)k] = scalp.normal[(size_t)t];
            }
        }
        std::vector<long long> keys(region);
        std::sort(keys.begin(), keys.end());
        keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
        work.resize(keys.size());
        for (size_t k = 0; k < rs.count(); ++k)
            work[std::lower_bound(keys.begin(), keys.end(), region[k]) - keys.begin()].push_back((uint32_t)k);
    } else {
        work.emplace_back(rs.count());
        std::iota(work[0].begin(), work[0].end(), 0u);
    }
    // top-down: each round fits every open cluster in parallel; coherent ones
    // become bundles, the others are split (order kept: deterministic)
    std::vector<std::vector<uint32_t>> done_members;
    std::vector<Fit> done_fits;
    while (!work.empty()) {
        std::vector<Fit> fits(work.size());
        std::vector<std::vector<uint32_t>> halves(2 * work.size());
#pragma omp parallel for schedule(dynamic, 1)
        for (long long i = 0; i < (long long)work.size(); ++i) {
            const auto& m = work[(size_t)i];
            if (m.size() > (size_t)kMaxMembers) {  // too large: split without fitting
                split_cluster(rs, m, halves[2 * i], halves[2 * i + 1]);
                continue;
            }
            fits[(size_t)i] = fit_cluster(cx, m);
            if (!fits[(size_t)i].coherent && m.size() > 1)
                split_cluster(rs, m, halves[2 * i], halves[2 * i + 1]);
        }
        std::vector<std::vector<uint32_t>> next;
        for (size_t i = 0; i < work.size(); ++i) {
            const bool fitted = work[i].size() <= (size_t)kMaxMembers;
            if (fitted && (fits[i].coherent || work[i].size() <= 1)) {
                done_members.push_back(std::move(work[i]));
                done_fits.push_back(std::move(fits[i]));
            } else {
                next.push_back(std::move(halves[2 * i]));
                next.push_back(std::move(halves[2 * i + 1]));
            }
        }
        work.swap(next);
    }
    // ambient occlusion per corner, then the buffers
    const size_t nb = done_fits.size();
    out->bundles.resize(nb);
    out->layers.resize(nb * kLayers * 4);
    out->style.resize(nb * kLayers * kTexels * 4);
    Density dens;
    const bool ao = (flags & HG_BAKE_AMBIENT_OCCLUSION) != 0;
    if (ao) dens = build_density(rs, cx.scalp);
#pragma omp parallel for schedule(dynamic, 16)
    for (long long bi = 0; bi < (long long)nb; ++bi) {
        const Cage& c = done_fits[(size_t)bi].cage;
        hg_gpu_bundle& b = out->bundles[(size_t)bi];
        b.layer_offset = (uint32_t)(bi * kLayers * 4);
        b.style_offset = (uint32_t)(bi * kLayers * kTexels);
        b.strand_count = (uint32_t)done_members[(size_t)bi].size();
        b.pad = 0;
        for (int l = 0; l < kLayers; ++l)
            for (int k = 0; k < 4; ++k) {
                const V3 p = c.q[l][k];
                const V3 prev = c.q[std::max(l - 1, 0)][k], next = c.q[std::min(l + 1, kLayers - 1)][k];
                const V3 tan = (l == 0 || l == kLayers - 1) ? next - prev : (next - prev) * 0.5f;
                const float occl = ao ? corner_ao(dens, p, unit_or(tan, {0.0f, 1.0f, 0.0f})) : 1.0f;
                hg_gpu_layer& g = out->layers[(size_t)b.layer_offset + l * 4 + k];
                g.pos_ao[0] = p.x, g.pos_ao[1] = p.y, g.pos_ao[2] = p.z, g.pos_ao[3] = occl;
                g.tangent[0] = tan.x, g.tangent[1] = tan.y, g.tangent[2] = tan.z, g.tangent[3] = 0.0f;
            }
        for (int t = 0; t < kLayers * kTexels; ++t) {
            float* s = &out->style[((size_t)b.style_offset + t) * 4];
            s[0] = c.style[t].x, s[1] = c.style[t].y, s[2] = c.style[t].z, s[3] = 0.0f;
        }
    }
    V3 lo{3e38f, 3e38f, 3e38f}, hi{-3e38f, -3e38f, -3e38f};
    for (const hg_gpu_layer& g : out->layers) {
        const V3 p{g.pos_ao[0], g.pos_ao[1], g.pos_ao[2]};
        lo = vmin(lo, p), hi = vmax(hi, p);
    }
    if (nb) {
        out->bounds[0] = lo.x, out->bounds[1] = lo.y, out->bounds[2] = lo.z;
        out->bounds[3] = hi.x, out->bounds[4] = hi.y, out->bounds[5] = hi.z;
    }
    return out;
}

}  // namespace

extern "C" {

hg_bake_result* hg_bake(const float* points, uint32_t n_points, const uint32_t* first, const uint32_t* count,
                        uint32_t n_strands, uint32_t flags) {
    return bake(points, n_points, first, count, n_strands, nullptr, 0, nullptr, 0, flags);
}

hg_bake_result* hg_bake_scalp(const float* points, uint32_t n_points, const uint32_t* first, const uint32_t* count,
                              uint32_t n_strands, const float* scalp_vertices, uint32_t n_scalp_vertices,
                              const uint32_t* scalp_indices, uint32_t n_scalp_indices, uint32_t flags) {
    return bake(points, n_points, first, count, n_strands, scalp_vertices, n_scalp_vertices, scalp_indices,
                n_scalp_indices, flags);
}

uint32_t hg_bake_bundle_count(const hg_bake_result* r) { return r ? (uint32_t)r->bundles.size() : 0u; }
uint32_t hg_bake_layer_count(const hg_bake_result* r) { return r ? (uint32_t)r->layers.size() : 0u; }
uint32_t hg_bake_style_count(const hg_bake_result* r) { return r ? (uint32_t)(r->style.size() / 4) : 0u; }

void hg_bake_copy(const hg_bake_result* r, hg_gpu_bundle* bundles, hg_gpu_layer* layers, float* style,
                  float bounds[6]) {
    if (!r) return;
    if (bundles && !r->bundles.empty()) std::memcpy(bundles, r->bundles.data(), r->bundles.size() * sizeof(hg_gpu_bundle));
    if (layers && !r->layers.empty()) std::memcpy(layers, r->layers.data(), r->layers.size() * sizeof(hg_gpu_layer));
    if (style && !r->style.empty()) std::memcpy(style, r->style.data(), r->style.size() * sizeof(float));
    if (bounds) std::memcpy(bounds, r->bounds, sizeof(r->bounds));
}

void hg_bake_free(hg_bake_result* r) { delete r; }

}  // extern "C"
