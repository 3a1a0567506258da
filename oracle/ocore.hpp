// ORACLE — test infrastructure only.  Nothing in the product (gammaray_gb300/) may
// include, link or call this code; only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg use it, and only as the checker.
//
// CPU restatement of the reference's src/core/ (sdao/gammaray, Rust): vector.rs, math.rs,
// ray.rs, bbox.rs, camera.rs, matrix.rs/xform.rs/quat.rs (the parts a camera needs) and
// random.rs.  Every function keeps the reference's order of float operations; the file
// is compiled with -ffp-contract=off because Rust never fuses a*b+c into an FMA.
//
// Parity unpinned: the reference ships no tests, golden vectors or fixtures, and cannot
// be built here (no Rust toolchain).  This restatement is checked in tests/ by analytic
// known-answer tests and physical invariants, against independent numpy restatements
// of the reference's code, and against golden vectors it wrote
// (tests/golden/oracle_golden.npz).  Those restatements cover the Disney material,
// intersection, shading frames, light sampling, camera and film.
//
// Random numbers.  The reference seeds XorShift from thread_rng (core/random.rs:13-20)
// and is not reproducible.  Here every random number is a pure function of
// (seed, pass, path, dimension), the same function the CUDA library uses, so both
// sides can be fed identical uniforms.  Samplers take their uniforms as arguments.
#pragma once

#include <cmath>
#include <cstdint>
#include <cfloat>
#include <vector>

namespace orc {

constexpr float EPS = FLT_EPSILON;               // std::f32::EPSILON
constexpr float PI = 3.14159265358979323846f;     // std::f32::consts::PI
constexpr float FRAC_1_PI = 0.318309886183790671538f;
constexpr float FRAC_PI_2 = 1.57079632679489661923f;
constexpr float FRAC_PI_4 = 0.785398163397448309616f;
constexpr float TWO_PI = 2.0f * PI;               // core/math.rs:3

// ---------------------------------------------------------------- core/math.rs
template <class T> inline T clamp(T x, T a, T b) {  // math.rs:5-15 (NaN passes through)
    if (x < a) return a;
    else if (x > b) return b;
    else return x;
}
inline float clamp_unit(float x) { return clamp(x, 0.0f, 1.0f); }
inline float lerp(float x, float y, float a) { return x + a * (y - x); }          // math.rs:22-24
inline float clamped_lerp(float x, float y, float a) { return lerp(x, y, clamp(a, 0.0f, 1.0f)); }
inline bool is_nearly_zero(float x) { return std::fabs(x) < EPS; }               // math.rs:37-39
inline bool is_positive(float x) { return x > EPS; }                             // math.rs:44-46
inline bool is_close(float x, float y, float eps) { return std::fabs(x - y) < eps; }
inline float gamma(float n) { return (n * EPS) / (1.0f - (n * EPS)); }           // math.rs:152-154

// math.rs:92-108, B = C = 1/3.
inline float mitchell_filter1(float x) {
    const float B = 1.0f / 3.0f;
    const float C = 1.0f / 3.0f;
    float twox = std::fabs(2.0f * x);
    if (twox > 1.0f) {
        return ((-B - 6.0f * C) * (twox * twox * twox)
                + (6.0f * B + 30.0f * C) * (twox * twox)
                + (-12.0f * B - 48.0f * C) * twox
                + (8.0f * B + 24.0f * C)) * (1.0f / 6.0f);
    } else {
        return ((12.0f - 9.0f * B - 6.0f * C) * (twox * twox * twox)
                + (-18.0f + 12.0f * B + 6.0f * C) * (twox * twox)
                + (6.0f - 2.0f * B)) * (1.0f / 6.0f);
    }
}
inline float mitchell_filter2(float x, float y, float width) {  // math.rs:121-123
    return mitchell_filter1(x / width) * mitchell_filter1(y / width);
}

// -------------------------------------------------------------- core/vector.rs
struct Vec {
    float x, y, z;
    Vec() : x(0), y(0), z(0) {}
    Vec(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    static Vec zero() { return Vec(0, 0, 0); }
    static Vec one() { return Vec(1, 1, 1); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    // vector.rs:21-24
    static Vec from_spherical(float cos_theta, float phi) {
        float sin_theta = std::sqrt(1.0f - cos_theta * cos_theta);
        return Vec(sin_theta * std::cos(phi), sin_theta * std::sin(phi), cos_theta);
    }
    Vec comp_mult(const Vec& o) const { return Vec(x * o.x, y * o.y, z * o.z); }
    Vec comp_div(const Vec& o) const { return Vec(x / o.x, y / o.y, z / o.z); }
    Vec cross(const Vec& o) const {  // vector.rs:45-50
        return Vec(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    float dot(const Vec& o) const { return x * o.x + y * o.y + z * o.z; }
    bool is_exactly_zero() const { return x == 0.0f && y == 0.0f && z == 0.0f; }
    bool is_close(const Vec& v, float eps) const {  // vector.rs:60-64
        return orc::is_close(v.x, x, eps) && orc::is_close(v.y, y, eps) && orc::is_close(v.z, z, eps);
    }
    float magnitude() const { return std::sqrt(dot(*this)); }
    Vec normalized() const {  // vector.rs:70-73: three divisions, not a reciprocal
        float length = magnitude();
        return Vec(x / length, y / length, z / length);
    }
    Vec sqrt() const { return Vec(std::sqrt(x), std::sqrt(y), std::sqrt(z)); }
    bool is_nearly_zero() const { return orc::is_nearly_zero(dot(*this)); }
    // vector.rs:91-104 (PBRT p. 63)
    void coord_system(Vec& v2, Vec& v3) const {
        if (std::fabs(x) > std::fabs(y)) {
            float inv_len = 1.0f / std::sqrt(x * x + z * z);
            v2 = Vec(-z * inv_len, 0.0f, x * inv_len);
        } else {
            float inv_len = 1.0f / std::sqrt(y * y + z * z);
            v2 = Vec(0.0f, z * inv_len, -y * inv_len);
        }
        v3 = cross(v2);
    }
    Vec world_to_local(const Vec& t, const Vec& b, const Vec& n) const {  // vector.rs:112-116
        return Vec(dot(t), dot(b), dot(n));
    }
    Vec local_to_world(const Vec& t, const Vec& b, const Vec& n) const {  // vector.rs:123-131
        return Vec(t.x * x + b.x * y + n.x * z,
                   t.y * x + b.y * y + n.y * z,
                   t.z * x + b.z * y + n.z * z);
    }
    float cos_theta() const { return z; }
    float cos2_theta() const { return z * z; }
    float abs_cos_theta() const { return std::fabs(z); }
    float sin2_theta() const { return std::fmax(0.0f, 1.0f - cos2_theta()); }
    float sin_theta() const { return std::sqrt(sin2_theta()); }
    float tan_theta() const { return sin_theta() / cos_theta(); }
    float tan2_theta() const { return sin2_theta() / cos2_theta(); }
    float cos_phi() const {  // vector.rs:175-183
        float sin_t = sin_theta();
        if (sin_t == 0.0f) return 1.0f;
        return clamp(x / sin_t, -1.0f, 1.0f);
    }
    float cos2_phi() const { return cos_phi() * cos_phi(); }
    float sin_phi() const {
        float sin_t = sin_theta();
        if (sin_t == 0.0f) return 0.0f;
        return clamp(y / sin_t, -1.0f, 1.0f);
    }
    float sin2_phi() const { return sin_phi() * sin_phi(); }
    bool is_local_same_hemisphere(const Vec& v) const { return z * v.z > 0.0f; }
    float luminance() const { return 0.21f * x + 0.71f * y + 0.08f * z; }  // vector.rs:218-220
    Vec tint() const {  // vector.rs:226-234
        float lume = luminance();
        if (lume > 0.0f) return Vec(x / lume, y / lume, z / lume);
        return one();
    }
    Vec reflect(const Vec& n) const {  // vector.rs:240-246
        float k = 2.0f * n.dot(*this);
        return Vec(n.x * k - x, n.y * k - y, n.z * k - z);
    }
    Vec refract(const Vec& n, float eta) const {  // vector.rs:253-264
        float cos_theta_in = n.dot(*this);
        float sin2_theta_in = std::fmax(0.0f, 1.0f - cos_theta_in * cos_theta_in);
        float sin2_theta_trans = eta * eta * sin2_theta_in;
        if (sin2_theta_trans >= 1.0f) return zero();
        float cos_theta_trans = std::sqrt(1.0f - sin2_theta_trans);
        Vec a(x * -eta, y * -eta, z * -eta);
        float k = eta * cos_theta_in - cos_theta_trans;
        return Vec(a.x + n.x * k, a.y + n.y * k, a.z + n.z * k);
    }
    bool is_finite() const { return std::isfinite(x) && std::isfinite(y) && std::isfinite(z); }
    Vec lerp(const Vec& o, float a) const {
        return Vec(orc::lerp(x, o.x, a), orc::lerp(y, o.y, a), orc::lerp(z, o.z, a));
    }
};
inline Vec operator+(const Vec& a, const Vec& b) { return Vec(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vec operator-(const Vec& a, const Vec& b) { return Vec(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vec operator*(const Vec& a, float k) { return Vec(a.x * k, a.y * k, a.z * k); }
inline Vec operator*(float k, const Vec& a) { return Vec(a.x * k, a.y * k, a.z * k); }
inline Vec operator/(const Vec& a, float k) { return Vec(a.x / k, a.y / k, a.z / k); }
inline Vec operator-(const Vec& a) { return Vec(-a.x, -a.y, -a.z); }

// ----------------------------------------------------------------- core/ray.rs
constexpr float RAY_PUSH_DIST = 1.0e-3f;  // ray.rs:9

struct Ray {
    Vec origin, direction;
    Ray() {}
    Ray(const Vec& o, const Vec& d) : origin(o), direction(d) {}
    Vec at(float k) const { return origin + (k * direction); }  // ray.rs:26-28
    Ray nudge() const { return Ray(origin + (direction * RAY_PUSH_DIST), direction); }
};

struct RayIntersectionData {  // ray.rs:31-42, 55-58
    Vec inv_dir;
    bool dir_is_neg[3];
    explicit RayIntersectionData(const Ray& r) {
        inv_dir = Vec(1.0f / r.direction.x, 1.0f / r.direction.y, 1.0f / r.direction.z);
        dir_is_neg[0] = r.direction.x < 0.0f;
        dir_is_neg[1] = r.direction.y < 0.0f;
        dir_is_neg[2] = r.direction.z < 0.0f;
    }
};

// ---------------------------------------------------------------- core/bbox.rs
struct BBox {
    Vec min, max;
    static BBox empty() {  // bbox.rs:14-19
        BBox b;
        b.min = Vec(FLT_MAX, FLT_MAX, FLT_MAX);
        b.max = Vec(-FLT_MAX, -FLT_MAX, -FLT_MAX);
        return b;
    }
    BBox union_with(const Vec& k) const {
        BBox b;
        b.min = Vec(std::fmin(min.x, k.x), std::fmin(min.y, k.y), std::fmin(min.z, k.z));
        b.max = Vec(std::fmax(max.x, k.x), std::fmax(max.y, k.y), std::fmax(max.z, k.z));
        return b;
    }
    BBox combine_with(const BBox& o) const {
        BBox b;
        b.min = Vec(std::fmin(min.x, o.min.x), std::fmin(min.y, o.min.y), std::fmin(min.z, o.min.z));
        b.max = Vec(std::fmax(max.x, o.max.x), std::fmax(max.y, o.max.y), std::fmax(max.z, o.max.z));
        return b;
    }
    Vec diagonal() const { return max - min; }
    // bbox.rs:44-56 — keeps the reference's test order (x wins only if y >= z too).
    int maximum_extent() const {
        Vec d = diagonal();
        if (d.x >= d.y && d.y >= d.z) return 0;
        else if (d.y >= d.z) return 1;
        else return 2;
    }
    Vec relative_offset(const Vec& v) const { return (v - min).comp_div(diagonal()); }
    // bbox.rs:73-76 — named surface_area but returns the volume (kept).
    float surface_area() const {
        Vec d = diagonal();
        return d.x * d.y * d.z;
    }
    const Vec& corner(bool is_max) const { return is_max ? max : min; }
    // bbox.rs:78-113 — slab test with gamma(3) inflation of the far distances.
    bool intersect(const Ray& ray, const RayIntersectionData& data, float max_dist) const {
        const float inflate = 1.0f + 2.0f * gamma(3.0f);
        float t_min = (corner(data.dir_is_neg[0]).x - ray.origin.x) * data.inv_dir.x;
        float t_max = (corner(!data.dir_is_neg[0]).x - ray.origin.x) * data.inv_dir.x;
        float ty_min = (corner(data.dir_is_neg[1]).y - ray.origin.y) * data.inv_dir.y;
        float ty_max = (corner(!data.dir_is_neg[1]).y - ray.origin.y) * data.inv_dir.y;
        t_max *= inflate;
        ty_max *= inflate;
        if (t_min > ty_max || ty_min > t_max) return false;
        if (ty_min > t_min) t_min = ty_min;
        if (ty_max < t_max) t_max = ty_max;
        float tz_min = (corner(data.dir_is_neg[2]).z - ray.origin.z) * data.inv_dir.z;
        float tz_max = (corner(!data.dir_is_neg[2]).z - ray.origin.z) * data.inv_dir.z;
        tz_max *= inflate;
        if (t_min > tz_max || tz_min > t_max) return false;
        if (tz_max < t_max) t_max = tz_max;
        return t_min < max_dist && t_max > 0.0f;
    }
};

// ------------------------------------------- core/matrix.rs, xform.rs, quat.rs
// Row-vector convention (v' = v * M, translation in row 3), xform.rs:41-54.
struct Mat {
    float m[4][4];
    static Mat identity() {
        Mat r;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) r.m[i][j] = (i == j) ? 1.0f : 0.0f;
        return r;
    }
    static Mat translation(const Vec& t) {  // matrix.rs:73-95
        Mat r = identity();
        r.m[3][0] = t.x;
        r.m[3][1] = t.y;
        r.m[3][2] = t.z;
        return r;
    }
    // matrix.rs:97-121 — rotation from a quaternion {real, i}.
    static Mat rotation(float rr, const Vec& i) {
        Mat o;
        o.m[0][0] = 1.0f - 2.0f * (i.y * i.y + i.z * i.z);
        o.m[0][1] = 2.0f * (i.x * i.y + i.z * rr);
        o.m[0][2] = 2.0f * (i.z * i.x - i.y * rr);
        o.m[0][3] = 0.0f;
        o.m[1][0] = 2.0f * (i.x * i.y - i.z * rr);
        o.m[1][1] = 1.0f - 2.0f * (i.z * i.z + i.x * i.x);
        o.m[1][2] = 2.0f * (i.y * i.z + i.x * rr);
        o.m[1][3] = 0.0f;
        o.m[2][0] = 2.0f * (i.z * i.x + i.y * rr);
        o.m[2][1] = 2.0f * (i.y * i.z - i.x * rr);
        o.m[2][2] = 1.0f - 2.0f * (i.y * i.y + i.x * i.x);
        o.m[2][3] = 0.0f;
        o.m[3][0] = 0.0f;
        o.m[3][1] = 0.0f;
        o.m[3][2] = 0.0f;
        o.m[3][3] = 1.0f;
        return o;
    }
    // Mat * Mat (matrix.rs Mul impl): plain row-by-column sum in index order.
    Mat operator*(const Mat& b) const {
        Mat r;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                float s = m[i][0] * b.m[0][j];
                s = s + m[i][1] * b.m[1][j];
                s = s + m[i][2] * b.m[2][j];
                s = s + m[i][3] * b.m[3][j];
                r.m[i][j] = s;
            }
        return r;
    }
    Vec transform(const Vec& v) const {  // xform.rs:41-47
        float x = v.x * m[0][0] + v.y * m[1][0] + v.z * m[2][0] + m[3][0];
        float y = v.x * m[0][1] + v.y * m[1][1] + v.z * m[2][1] + m[3][1];
        float z = v.x * m[0][2] + v.y * m[1][2] + v.z * m[2][2] + m[3][2];
        float w = v.x * m[0][3] + v.y * m[1][3] + v.z * m[2][3] + m[3][3];
        return Vec(x / w, y / w, z / w);
    }
    Vec transform_dir(const Vec& v) const {  // xform.rs:49-54
        return Vec(v.x * m[0][0] + v.y * m[1][0] + v.z * m[2][0],
                   v.x * m[0][1] + v.y * m[1][1] + v.z * m[2][1],
                   v.x * m[0][2] + v.y * m[1][2] + v.z * m[2][2]);
    }
};

// -------------------------------------------------------------- core/camera.rs
struct Camera {
    float focal_length, horizontal_aperture, vertical_aperture, f_stop;
    Mat xform;
    // camera.rs:42-61: xform = translation * rotation.
    Camera(float f, float h_ap, float v_ap, float fstop, float q_real, const Vec& q_imag,
           const Vec& translate)
        : focal_length(f), horizontal_aperture(h_ap), vertical_aperture(v_ap), f_stop(fstop) {
        xform = Mat::translation(translate) * Mat::rotation(q_real, q_imag);
    }
    void window_max(float& wx, float& wy) const {  // camera.rs:76-79
        wx = horizontal_aperture / (focal_length * 2.0f);
        wy = vertical_aperture / (focal_length * 2.0f);
    }
    Ray compute_ray(float s, float t) const {  // camera.rs:87-97
        float wx, wy;
        window_max(wx, wy);
        Vec origin = Vec::zero();
        Vec direction = Vec(wx * s, wy * t, -1.0f).normalized();
        return Ray(xform.transform(origin), xform.transform_dir(direction));
    }
};

// ---------------------------------------------------------- random numbers
// Counter-based stream shared with the CUDA library: a SplitMix64 finaliser
// (Steele, Lea & Flood 2014) keyed on (seed, pass, path) and indexed by dimension.
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t path_key(uint64_t seed, uint32_t pass, uint32_t path) {
    return mix64(seed ^ mix64((static_cast<uint64_t>(pass) << 32) | path));
}
inline float uniform(uint64_t key, uint32_t dim) {  // [0, 1) with 24 random bits
    uint64_t h = mix64(key + static_cast<uint64_t>(dim) * 0xD1B54A32D192ED03ull);
    return static_cast<float>(static_cast<uint32_t>(h >> 40)) * (1.0f / 16777216.0f);
}

// A stream view of one path: dimension `base + k` for the k-th draw of a step.
struct Sampler {
    uint64_t key;
    uint32_t base;
    uint32_t used;
    Sampler(uint64_t k, uint32_t b) : key(k), base(b), used(0) {}
    float next_f32() { return uniform(key, base + used++); }
};

// Dimension layout of one camera path (both libraries use the same layout).
constexpr uint32_t DIM_JITTER_ROW = 0;
constexpr uint32_t DIM_JITTER_COL = 1;
constexpr uint32_t DIM_CAMERA_WALK = 2;   // + 4 * vertex: lobe, u1, u2, roulette
constexpr uint32_t DIM_LIGHT_SAMPLE = 66; // light, component, area u1, u2, dir u1, u2
constexpr uint32_t DIM_LIGHT_WALK = 72;   // + 4 * vertex

// rand::distributions::Range<usize>::new(0, n) replaced by a uniform index.
inline uint32_t range_index(float u, uint32_t n) {
    uint32_t i = static_cast<uint32_t>(u * static_cast<float>(n));
    return i < n ? i : n - 1;
}

// -------------------------------------------------------------- core/random.rs
// AreaSampleDisk (random.rs:28-56): two Range(-1, 1) draws.
inline void area_sample_disk(float u1, float u2, float& dx, float& dy) {
    float sx = -1.0f + 2.0f * u1;
    float sy = -1.0f + 2.0f * u2;
    if (sx == 0.0f && sy == 0.0f) {
        dx = 0.0f;
        dy = 0.0f;
        return;
    }
    float r, theta;
    if (std::fabs(sx) > std::fabs(sy)) {
        r = sx;
        theta = FRAC_PI_4 * (sy / sx);
    } else {
        r = sy;
        theta = FRAC_PI_2 - FRAC_PI_4 * (sx / sy);
    }
    dx = r * std::cos(theta);
    dy = r * std::sin(theta);
}
// CosineSampleHemisphere (random.rs:70-106).
inline Vec cosine_sample_hemisphere(bool flipped, float u1, float u2) {
    float x, y;
    area_sample_disk(u1, u2, x, y);
    float z = std::sqrt(std::fmax(0.0f, 1.0f - x * x - y * y));
    if (flipped) return Vec(x, y, -1.0f * z);
    return Vec(x, y, z);
}
inline float cosine_hemisphere_pdf(const Vec& d) { return d.abs_cos_theta() * FRAC_1_PI; }
// UniformSampleSphere (random.rs:113-148).  The reference normalises three normal
// deviates from rand's Ziggurat; here the same uniform-on-sphere law is drawn by
// inversion (z = 1 - 2 u1, phi = 2 pi u2) from two uniforms.
inline Vec uniform_sample_sphere(float u1, float u2) {
    float z = 1.0f - 2.0f * u1;
    float r = std::sqrt(std::fmax(0.0f, 1.0f - z * z));
    float phi = TWO_PI * u2;
    return Vec(r * std::cos(phi), r * std::sin(phi), z);
}
// UniformSampleBarycentric (random.rs:258-274).
inline void uniform_sample_barycentric(float a, float b, float& u, float& v) {
    float sqrt_a = std::sqrt(a);
    u = 1.0f - sqrt_a;
    v = b * sqrt_a;
}
// CumulativeDistribution::ind_sample (random.rs:232-256): binary search of the target.
inline size_t cdf_sample(const std::vector<float>& cdf, float target) {
    size_t lo = 0, hi = cdf.size();
    while (lo < hi) {
        size_t mid = lo + (hi - lo) / 2;
        if (cdf[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

}  // namespace orc
