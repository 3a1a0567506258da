// Closest-hit and shadow traversal of the wide BVH (replaces Bvh::intersect,
// geom/bvh.rs:406-456, and Bvh::visibility, bvh.rs:460-477).
//
// One thread per ray.  A node is 2W float4s (W = 2, 4, 8) read with vector loads;
// every child box is slab-tested (far distances inflated by 1 + 2 gamma(3) as in
// core/bbox.rs:78-113), the hit children are ordered near-to-far by a sorting network
// on (distance | slot) keys, and the farther ones go on a per-thread stack of
// (child, entry distance) pairs: the first SMEM_STACK entries in shared memory, column
// `threadIdx.x`, deeper ones in a local array.  Popped entries whose entry distance is
// no longer below the closest hit are skipped.  Every traversal (closest hit, shadow
// rays, query kernels) runs the step functions below; visit_node and visit_leaf are the
// only node and leaf tests.
// Leaves hold up to 16 consecutive primitive records.  The primitive tests are the
// reference's Moller-Trumbore (geom/mesh.rs:270-308) and sphere quadratic
// (geom/sphere.rs:70-101) with the same operation order, so a hit distance is
// bit-identical to the reference's for the same triangle.
#pragma once

#include "scene.hpp"

namespace gr {

struct TraceResult {
    float t;
    int32_t k;  // leaf-order primitive index, -1 = miss
    float u, v;
};

// Reference primitive tests.  Returns the distance (0 = miss).
GR_D float intersect_prim(const float4 p0, const float4 p1, const float4 p2, V3 o, V3 d, float& uo, float& vo) {
    if (__float_as_int(p2.w) == PRIM_TRIANGLE) {
        V3 c = V3{p0.x, p0.y, p0.z};
        V3 e1 = V3{p1.x, p1.y, p1.z};
        V3 e2 = V3{p2.x, p2.y, p2.z};
        V3 p = cross(d, e2);
        float det = dot(e1, p);
        if (nearly_zero(det)) return 0.0f;
        float inv_det = 1.0f / det;
        V3 t = o - c;
        float u = dot(t, p) * inv_det;
        if (u < 0.0f || u > 1.0f) return 0.0f;
        V3 q = cross(t, e1);
        float v = dot(d, q) * inv_det;
        if (v < 0.0f || (u + v) > 1.0f) return 0.0f;
        float dist = dot(e2, q) * inv_det;
        if (!is_positive(dist)) return 0.0f;
        uo = u;
        vo = v;
        return dist;
    }
    V3 oc = o - V3{p0.x, p0.y, p0.z};
    float r = p1.x;
    float a = dot(d, d);
    float b = dot(d, oc);
    float c = dot(oc, oc) - (r * r);
    float disc = (b * b) - (a * c);
    if (disc > 0.0f) {
        float sq = sqrtf(disc);
        float res_pos = -b + sq;
        float res_neg = -b - sq;
        if (is_positive(res_neg)) return res_neg;
        if (is_positive(res_pos)) return res_pos;
    }
    return 0.0f;
}

// child[slot] without dynamic register indexing (keeps the node in registers).
template <int W>
GR_D int32_t select_child(const float (&f)[8 * W], uint32_t slot) {
    if (W == 4) {  // by the slot's two bits: three selects
        const float lo = (slot & 1u) ? f[6 * W + 1] : f[6 * W];
        const float hi = (slot & 1u) ? f[6 * W + 3] : f[6 * W + 2];
        return __float_as_int((slot & 2u) ? hi : lo);
    }
    int32_t r = 0;
#pragma unroll
    for (int j = 0; j < W; ++j)
        if (static_cast<uint32_t>(j) == slot) r = __float_as_int(f[6 * W + j]);
    return r;
}

template <int N>
GR_D void sort_keys(uint32_t (&k)[N]) {
    if (N == 4) {  // the 5-comparator network for 4 keys
        const int pairs[5][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}, {1, 2}};
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            uint32_t a = k[pairs[c][0]], b = k[pairs[c][1]];
            k[pairs[c][0]] = min(a, b);
            k[pairs[c][1]] = max(a, b);
        }
        return;
    }
    // Odd-even transposition network, fully unrolled (N <= 8).
#pragma unroll
    for (int pass = 0; pass < N; ++pass) {
#pragma unroll
        for (int i = pass & 1; i + 1 < N; i += 2) {
            uint32_t a = k[i], b = k[i + 1];
            k[i] = min(a, b);
            k[i + 1] = max(a, b);
        }
    }
}

}  // namespace gr

namespace gr {

// ---------------------------------------------------------------------------
// Step-wise traversal for the persistent extension kernel.  The state of one ray lives
// in registers; trav_step() processes one interior node or one leaf.  The stack keeps
// its first SMEM_STACK entries in this thread's shared-memory column and spills deeper
// entries to a per-thread local array (rarely touched, cached in L1), so the shared
// footprint no longer scales with the tree's worst-case depth.
// Stack entries per thread kept in shared memory (MAX_STACK in common.cuh: both builds
// reject deeper trees); deeper entries go to the local spill array.  On the path-tracer
// workload (102,422 triangles, 1024 x 1024, 64 spp) 4 / 8 / 12 / 16 measured 1863 /
// 1883 / 1887 / 1881 Msamples/s: the L1 left to node and primitive loads by a smaller
// shared part does not matter.
#ifndef GR_SMEM_STACK
#define GR_SMEM_STACK 16
#endif
constexpr int SMEM_STACK = GR_SMEM_STACK;
static_assert(SMEM_STACK >= 1 && SMEM_STACK <= MAX_STACK, "shared stack part within the stack bound");

// Extension kernels that refill their warps (k_extend_refill, k_eng_extend_refill): a
// warp takes new rays for its idle lanes once at least this many are idle; 0 selects the
// kernels with one ray per thread and no refill.  On the path-tracer workload (102,422
// triangles, 1024 x 1024, 64 spp) 0 / 4 / 8 / 16 measured 1298 / 1511 / 1565 / 1586
// Msamples/s.
#ifndef GR_EXTEND_REFILL
#define GR_EXTEND_REFILL 16
#endif

// The two arrays a traversal step reads.  A kernel whose lanes trace rays of different
// scenes keeps one per lane in registers instead of reloading them through a scene
// record at every step.
struct TraceScene {
    const float4* nodes;
    const float4* prims;
};

struct TravState {
    V3 o, d, inv;
    float closest;
    float hu, hv;
    int32_t ref;
    int32_t hit;
    int sp;
    bool nx, ny, nz;
};

GR_D void trav_init(TravState& t, V3 o, V3 d, float t_max) {
    t.o = o;
    t.d = d;
    t.inv = V3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    t.nx = d.x < 0.0f;
    t.ny = d.y < 0.0f;
    t.nz = d.z < 0.0f;
    t.closest = t_max;
    t.hu = t.hv = 0.0f;
    t.ref = 0;
    t.hit = -1;
    t.sp = 0;
}

// Stack entries are (child reference, entry distance bits) pairs, one 64-bit access each.
struct StackView {
    int2* s;      // this thread's shared column (stride = blockDim.x entries)
    int stride;
    int2* spill;  // local overflow, MAX_STACK - SMEM_STACK entries
    GR_D void push(int sp, int32_t ref, float te) const {
        const int2 e = make_int2(ref, __float_as_int(te));
        if (sp < SMEM_STACK) s[sp * stride] = e;
        else spill[sp - SMEM_STACK] = e;
    }
    GR_D void pop(int sp, int32_t& ref, float& te) const {
        int2 e;
        if (sp < SMEM_STACK) e = s[sp * stride];  // shared and local loads kept apart
        else e = spill[sp - SMEM_STACK];
        ref = e.x;
        te = __int_as_float(e.y);
    }
};

// Tests one wide node against the ray: pushes the far hit children (sorted by entry
// distance, nearest last) and makes the nearest hit child the current reference.
// Returns false when no child is hit.  A push beyond MAX_STACK sets *err = 1 and
// `overflow`.
template <int W, bool COUNT, class S>
GR_D bool visit_node(const S& s, TravState& t, const StackView& stk, int* err, uint32_t* counts,
                     bool& overflow) {
    const float inflate = 1.0f + 2.0f * gamma_n(3.0f);
    if (COUNT) counts[0] += 1;
    const float4* nb = s.nodes + static_cast<size_t>(t.ref) * (2 * W);
    // f holds the rows lo_x lo_y lo_z hi_x hi_y hi_z child (W floats each).  With W a
    // multiple of 4 a row is whole float4s, so the ray loads its near and far planes
    // straight into the lo and hi rows (row offsets from its direction signs) and skips
    // the padding row: no per-child selects, one load fewer.  The arithmetic is the same
    // as selecting them.
    float f[8 * W];
    if (W % 4 == 0) {
        constexpr int R = W / 4;  // float4 per row
        const int rows[7] = {t.nx ? 3 : 0, t.ny ? 4 : 1, t.nz ? 5 : 2, t.nx ? 0 : 3, t.ny ? 1 : 4, t.nz ? 2 : 5, 6};
#pragma unroll
        for (int r = 0; r < 7; ++r)
#pragma unroll
            for (int q = 0; q < R; ++q) {
                float4 x = __ldg(nb + rows[r] * R + q);
                f[r * W + 4 * q] = x.x;
                f[r * W + 4 * q + 1] = x.y;
                f[r * W + 4 * q + 2] = x.z;
                f[r * W + 4 * q + 3] = x.w;
            }
    } else {
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) {
            float4 x = __ldg(nb + q);
            f[4 * q] = x.x;
            f[4 * q + 1] = x.y;
            f[4 * q + 2] = x.z;
            f[4 * q + 3] = x.w;
        }
    }
    uint32_t key[W];
    int h = 0;
#pragma unroll
    for (int j = 0; j < W; ++j) {
        float t0x, t1x, t0y, t1y, t0z, t1z;
        if (W % 4 == 0) {  // rows 0-2 near, 3-5 far
            t0x = (f[0 * W + j] - t.o.x) * t.inv.x;
            t0y = (f[1 * W + j] - t.o.y) * t.inv.y;
            t0z = (f[2 * W + j] - t.o.z) * t.inv.z;
            t1x = (f[3 * W + j] - t.o.x) * t.inv.x;
            t1y = (f[4 * W + j] - t.o.y) * t.inv.y;
            t1z = (f[5 * W + j] - t.o.z) * t.inv.z;
        } else {
            float lx = f[0 * W + j], ly = f[1 * W + j], lz = f[2 * W + j];
            float hx = f[3 * W + j], hy = f[4 * W + j], hz = f[5 * W + j];
            t0x = ((t.nx ? hx : lx) - t.o.x) * t.inv.x;
            t1x = ((t.nx ? lx : hx) - t.o.x) * t.inv.x;
            t0y = ((t.ny ? hy : ly) - t.o.y) * t.inv.y;
            t1y = ((t.ny ? ly : hy) - t.o.y) * t.inv.y;
            t0z = ((t.nz ? hz : lz) - t.o.z) * t.inv.z;
            t1z = ((t.nz ? lz : hz) - t.o.z) * t.inv.z;
        }
        float tmin = fmaxf(fmaxf(t0x, t0y), t0z);
        float tmax = fminf(fminf(t1x, t1y), t1z) * inflate;
        // The slab test (tmin <= tmax, tmax > 0, tmin < closest) on te = max(tmin, 0):
        // the same result (closest > 0), except that a box whose far distance is exactly
        // 0 counts as hit, which can only add a node to visit.
        float te = fmaxf(tmin, 0.0f);
        bool hit = te <= tmax && te < t.closest;
        key[j] = hit ? ((__float_as_uint(te) & ~7u) | static_cast<uint32_t>(j)) : 0xFFFFFFFFu;
        h += hit ? 1 : 0;
    }
    if (h == 0) return false;
    sort_keys<W>(key);
    if (t.sp + h - 1 > MAX_STACK) {
        *err = 1;
        overflow = true;
        return false;
    }
#pragma unroll
    for (int j = W - 1; j >= 1; --j) {
        if (j < h) {
            stk.push(t.sp, select_child<W>(f, key[j] & 7u), __uint_as_float(key[j] & ~7u));
            ++t.sp;
        }
    }
    t.ref = select_child<W>(f, key[0] & 7u);
    return true;
}

// Intersects the primitives of leaf `ref`, keeping the closest hit in t.  With ANY_HIT
// it returns true at the first hit closer than t.closest.
template <bool ANY_HIT, bool COUNT, class S>
GR_D bool visit_leaf(const S& s, TravState& t, int32_t ref, uint32_t* counts) {
    uint32_t enc = ~static_cast<uint32_t>(ref);
    uint32_t first = enc >> LEAF_COUNT_BITS;
    uint32_t count = (enc & (MAX_LEAF_PRIMS - 1)) + 1;
    if (COUNT) counts[1] += count;
    for (uint32_t k = first; k < first + count; ++k) {
        const float4* pr = s.prims + 3 * static_cast<size_t>(k);
        float4 p0 = __ldg(pr), p1 = __ldg(pr + 1), p2 = __ldg(pr + 2);
        float u, v;
        float dist = intersect_prim(p0, p1, p2, t.o, t.d, u, v);
        if (dist != 0.0f && dist < t.closest) {
            t.closest = dist;
            t.hit = static_cast<int32_t>(k);
            t.hu = u;
            t.hv = v;
            if (ANY_HIT) return true;
        }
    }
    return false;
}

// Pops the next stacked child that can still hold a closer hit into t.ref.  Returns
// false when the stack is exhausted.
GR_D bool pop_next(TravState& t, const StackView& stk) {
    while (t.sp > 0) {
        --t.sp;
        int32_t r;
        float te;
        stk.pop(t.sp, r, te);
        if (te < t.closest) {
            t.ref = r;
            return true;
        }
    }
    return false;
}

// One traversal step.  Returns true when the ray is finished (t.hit / t.closest hold
// the closest hit).  With ANY_HIT it finishes at the first hit closer than t_max.
// S is DeviceScene or TraceScene: the step functions read only `nodes` and `prims`.
template <int W, bool ANY_HIT, bool COUNT, class S>
GR_D bool trav_step(const S& s, TravState& t, const StackView& stk, int* err, uint32_t* counts) {
    if (t.ref >= 0) {
        bool overflow = false;
        bool descended = visit_node<W, COUNT>(s, t, stk, err, counts, overflow);
        if (overflow) {
            t.hit = -1;
            return true;
        }
        if (descended) return false;
    } else if (visit_leaf<ANY_HIT, COUNT>(s, t, t.ref, counts)) {
        return true;
    }
    return !pop_next(t, stk);
}

inline size_t step_stack_smem_bytes(int threads) {
    return static_cast<size_t>(SMEM_STACK) * threads * (sizeof(int32_t) + sizeof(float));
}

// A thread's traversal stack: its column of the block's shared stack (dynamic shared
// memory starting at `smem`, step_stack_smem_bytes(blockDim.x) bytes) and its local
// spill array.
GR_D StackView thread_stack(unsigned char* smem, int2* spill) {
    return StackView{reinterpret_cast<int2*>(smem) + threadIdx.x, static_cast<int>(blockDim.x), spill};
}

// Traces one ray to the end.  ANY_HIT: stops at the first hit closer than t_max (shadow
// rays).  A miss returns t = t_max and k = -1.  A ray that needs more than the scene's
// step budget is abandoned as a miss and flagged: *err = 2 and, if err_ray is given, the
// ray's index there.  A stack overflow (impossible for trees the builds accept) sets
// *err = 1.  With COUNT, counts[0] / counts[1] accumulate nodes visited / primitives
// tested.
template <int W, bool ANY_HIT, bool COUNT = false>
GR_D TraceResult trace_ray(const DeviceScene& s, V3 o, V3 d, float t_max, const StackView& stk, int* err,
                           int* err_ray = nullptr, uint32_t ray = 0, uint32_t* counts = nullptr) {
    TravState t;
    trav_init(t, o, d, t_max);
    uint32_t steps = 0;
    while (!trav_step<W, ANY_HIT, COUNT>(s, t, stk, err, counts)) {
        if (++steps > s.step_budget) {
            atomicExch(err, 2);
            if (err_ray) atomicExch(err_ray, static_cast<int>(ray));
            return TraceResult{t_max, -1, 0.0f, 0.0f};
        }
    }
    return TraceResult{t.closest, t.hit, t.hu, t.hv};
}

}  // namespace gr
