// Shared device/host definitions of the GB300 rendering library.
//
// Float arithmetic follows the reference's order of operations, and the library is
// compiled with -fmad=false (device) and -ffp-contract=off (host) so that a*b+c stays
// two rounded operations as in Rust.  Division and sqrt are IEEE (nvcc defaults
// -prec-div=true, -prec-sqrt=true); no fast-math anywhere.
#pragma once

#include <cfloat>
#include <cstdint>
#include <math.h>
#include <cuda_runtime.h>

#define GR_HD __host__ __device__ __forceinline__
#define GR_D __device__ __forceinline__

// Checked build (-DGR_CHECKED=1, the stand-in for a memory checker): every queue, entry
// and shadow-queue write tests its index against its buffer's capacity, skips the write
// when it is out of range and sets this file's flag, which the host reads after the
// render (GR_ERR_INTERNAL).  Off by default; then GR_IN_RANGE is `true`.
#ifndef GR_CHECKED
#define GR_CHECKED 0
#endif

namespace gr {

#if GR_CHECKED && defined(__CUDACC__)
static __device__ unsigned int g_bad_index = 0u;
#define GR_IN_RANGE(i, n) ((i) < (n) || (atomicExch(&g_bad_index, 1u), false))
// Reads and clears this file's flag (host).
static inline cudaError_t take_bad_index(bool& bad) {
    unsigned int v = 0u, z = 0u;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_bad_index, sizeof(v));
    if (e == cudaSuccess && v) e = cudaMemcpyToSymbol(g_bad_index, &z, sizeof(z));
    bad = v != 0u;
    return e;
}
#else
#define GR_IN_RANGE(i, n) true
#endif

constexpr float EPS = FLT_EPSILON;
constexpr float PI = 3.14159265358979323846f;
constexpr float FRAC_1_PI = 0.318309886183790671538f;
constexpr float FRAC_PI_2 = 1.57079632679489661923f;
constexpr float FRAC_PI_4 = 0.785398163397448309616f;
constexpr float TWO_PI = 2.0f * PI;
constexpr float RAY_PUSH_DIST = 1.0e-3f;
constexpr uint32_t NO_INDEX = 0xFFFFFFFFu;

struct V3 {
    float x, y, z;
};

GR_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
GR_HD V3 v3zero() { return V3{0.0f, 0.0f, 0.0f}; }
GR_HD V3 v3one() { return V3{1.0f, 1.0f, 1.0f}; }
GR_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
GR_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
GR_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
GR_HD V3 operator*(V3 a, float k) { return V3{a.x * k, a.y * k, a.z * k}; }
GR_HD V3 operator*(float k, V3 a) { return V3{a.x * k, a.y * k, a.z * k}; }
GR_HD V3 operator/(V3 a, float k) { return V3{a.x / k, a.y / k, a.z / k}; }
GR_HD V3 mul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
GR_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GR_HD V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
GR_HD bool is_zero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
GR_HD float magnitude(V3 a) { return sqrtf(dot(a, a)); }
GR_HD V3 normalized(V3 a) {  // three divisions, as the reference (core/vector.rs:70-73)
    float l = magnitude(a);
    return V3{a.x / l, a.y / l, a.z / l};
}
GR_HD V3 vsqrt(V3 a) { return V3{sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)}; }
GR_HD bool nearly_zero(float x) { return fabsf(x) < EPS; }
GR_HD bool nearly_zero(V3 a) { return nearly_zero(dot(a, a)); }
GR_HD bool is_positive(float x) { return x > EPS; }
GR_HD float lerp(float x, float y, float a) { return x + a * (y - x); }

// Division of 32-bit unsigned integers by a divisor fixed for a launch (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994): with
// l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1, floor(n / d) is
// (t + ((n - t) >> 1)) >> (l - 1) for t = mulhi(m, n), exact for every n and 1 <= d < 2^31.
struct FastDiv {
    uint32_t d = 1, m = 0, l = 0;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    if (d > 1) {
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;
        f.l = l;
        f.m = static_cast<uint32_t>(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
    return f;
}
GR_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return static_cast<uint32_t>((static_cast<uint64_t>(a) * b) >> 32);
#endif
}
GR_HD uint32_t fast_div(uint32_t n, const FastDiv& f) {
    if (f.d == 1) return n;
    const uint32_t t = mulhi32(f.m, n);
    return (t + ((n - t) >> 1)) >> (f.l - 1);
}
GR_HD V3 vlerp(V3 a, V3 b, float t) { return V3{lerp(a.x, b.x, t), lerp(a.y, b.y, t), lerp(a.z, b.z, t)}; }
GR_HD float clampf(float x, float a, float b) { return x < a ? a : (x > b ? b : x); }  // NaN passes through
GR_HD float clamp_unit(float x) { return clampf(x, 0.0f, 1.0f); }
GR_HD float clamped_lerp(float x, float y, float a) { return lerp(x, y, clampf(a, 0.0f, 1.0f)); }
GR_HD float luminance(V3 c) { return 0.21f * c.x + 0.71f * c.y + 0.08f * c.z; }
GR_HD V3 tint(V3 c) {
    float l = luminance(c);
    return l > 0.0f ? V3{c.x / l, c.y / l, c.z / l} : v3one();
}
GR_HD float gamma_n(float n) { return (n * EPS) / (1.0f - (n * EPS)); }

// core/vector.rs:91-104 (PBRT p. 63)
GR_HD void coord_system(V3 v, V3& v2, V3& v3o) {
    if (fabsf(v.x) > fabsf(v.y)) {
        float inv_len = 1.0f / sqrtf(v.x * v.x + v.z * v.z);
        v2 = V3{-v.z * inv_len, 0.0f, v.x * inv_len};
    } else {
        float inv_len = 1.0f / sqrtf(v.y * v.y + v.z * v.z);
        v2 = V3{0.0f, v.z * inv_len, -v.y * inv_len};
    }
    v3o = cross(v, v2);
}
GR_HD V3 world_to_local(V3 v, V3 t, V3 b, V3 n) { return V3{dot(v, t), dot(v, b), dot(v, n)}; }
GR_HD V3 local_to_world(V3 v, V3 t, V3 b, V3 n) {
    return V3{t.x * v.x + b.x * v.y + n.x * v.z, t.y * v.x + b.y * v.y + n.y * v.z, t.z * v.x + b.z * v.y + n.z * v.z};
}

// SurfaceProperties (geom/prim.rs:57-79)
struct Frame {
    V3 normal, tangent, binormal, geom_normal;
};

// ---------------------------------------------------------------- random numbers
// Counter-based: a SplitMix64 finaliser (Steele, Lea & Flood 2014) keyed on
// (seed, pass, path) and indexed by dimension; identical on host and device.
GR_HD uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
GR_HD uint64_t path_key(uint64_t seed, uint32_t pass, uint32_t path) {
    return mix64(seed ^ mix64((static_cast<uint64_t>(pass) << 32) | path));
}
GR_HD float uniform01(uint64_t key, uint32_t dim) {
    uint64_t h = mix64(key + static_cast<uint64_t>(dim) * 0xD1B54A32D192ED03ull);
    return static_cast<float>(static_cast<uint32_t>(h >> 40)) * (1.0f / 16777216.0f);
}
GR_HD uint32_t range_index(float u, uint32_t n) {
    uint32_t i = static_cast<uint32_t>(u * static_cast<float>(n));
    return i < n ? i : n - 1;
}

// Dimension layout of one camera path (same on every backend).
constexpr uint32_t DIM_JITTER_ROW = 0;
constexpr uint32_t DIM_JITTER_COL = 1;
constexpr uint32_t DIM_CAMERA_WALK = 2;   // + 4 * vertex: lobe, u1, u2, roulette
constexpr uint32_t DIM_LIGHT_SAMPLE = 66; // light, component, area u1, u2, dir u1, u2
constexpr uint32_t DIM_LIGHT_WALK = 72;   // + 4 * vertex

// ------------------------------------------------------------------- layouts

// Lobe kinds (material/lobes.rs:25-40).
enum : uint32_t {
    LOBE_NONE = 0,
    LOBE_DIFFUSE = 1,
    LOBE_SPECULAR = 2,
    LOBE_GLOSSY = 4,
    LOBE_REFLECTION = 8,
    LOBE_TRANSMISSION = 16,
};

enum LobeType : int32_t {
    L_DISNEY_DIFFUSE = 0,   // lobes.rs:76-116
    L_GGX_DISNEY = 1,       // StandardMicrofacetRefl<GGX, DisneyFresnel>, lobes.rs:212-226
    L_GTR1_SCHLICK = 2,     // StandardMicrofacetRefl<GTR1, Schlick>, lobes.rs:228-243
    L_SPECULAR_TRANS = 3,   // lobes.rs:246-393
    L_PERFECT_DIFFUSE = 4,  // lobes.rs:401-414
    L_PERFECT_MIRROR = 5,   // lobes.rs:422-457
};

// One lobe with its constructor-time constants already evaluated on the host.
//   DISNEY_DIFFUSE: c0 = colour, c1 = sheen colour, p[0] = roughness
//   GGX_DISNEY:     c0 = base colour (conductor), c1 = specular colour, p = ax, ay, ior, metallic
//   GTR1_SCHLICK:   c0 = lobe colour (0.25 clearcoat), c1 = r0, p[0] = alpha
//   SPECULAR_TRANS: c0 = colour, p = ax, ay, ior
struct alignas(16) DevLobe {
    int32_t type;
    uint32_t kind;
    float c0[3];
    float c1[3];
    float p[4];
};

constexpr int MAX_LOBES = 4;

struct alignas(16) DevMaterial {
    int32_t n_lobes;
    int32_t has_light;
    float emission[3];
    float display[3];
    uint32_t lobe_set;  // n_lobes and the lobe types, 3 bits each (the shading sort's key)
    DevLobe lobe[MAX_LOBES];
};

// Primitive record in leaf order, 48 bytes:
//   triangle: p0 = (c, prim), p1 = (a - c, component), p2 = (b - c, 0)
//   sphere:   p0 = (centre, prim), p1 = (radius, 0, 0, 0), p2 = (0, 0, 0, 1)
constexpr int PRIM_TRIANGLE = 0;
constexpr int PRIM_SPHERE = 1;

// Leaf reference in a wide node child slot: child < 0, ~child = (first << 4) | (count - 1).
constexpr int LEAF_COUNT_BITS = 4;
// Traversal stack entries a ray may need (the tree's worst case); the host and device
// builds reject trees that exceed it.
constexpr int MAX_STACK = 96;
constexpr int MAX_LEAF_PRIMS = 1 << LEAF_COUNT_BITS;

}  // namespace gr
