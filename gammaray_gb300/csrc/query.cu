// Batched queries behind gr_trace_rays / gr_intersect_naive / gr_visibility /
// gr_sample_light / gr_bsdf_*: one thread per query, used by the parity tests and by
// callers that bring their own rays.
#include "runtime.hpp"
#include "traverse.cuh"

namespace gr {

namespace {

constexpr int QUERY_BLOCK = 128;

GR_D void write_hit(const DeviceScene& s, gr_hit* out, const TraceResult& r) {
    gr_hit h;
    if (r.k < 0) {
        h.t = 0.0f;
        h.prim = -1;
        h.component = -1;
        h.u = h.v = 0.0f;
    } else {
        const float4* pr = s.prims + 3 * static_cast<size_t>(r.k);
        h.t = r.t;
        h.prim = __float_as_int(__ldg(pr).w);
        h.component = __float_as_int(__ldg(pr + 1).w);
        h.u = r.u;
        h.v = r.v;
    }
    *out = h;
}

template <int W, bool ANY>
__global__ void __launch_bounds__(QUERY_BLOCK) k_trace(DeviceScene s, const float* __restrict__ rays, uint64_t n,
                                                       gr_hit* __restrict__ hits, const float* __restrict__ tmax,
                                                       int* err) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + 6 * i;
    V3 o = V3{r[0], r[1], r[2]};
    V3 d = V3{r[3], r[4], r[5]};
    float tm = tmax ? tmax[i] : FLT_MAX;
    TraceResult res = trace_ray<W, ANY>(s, o, d, tm, stk, err);
    write_hit(s, hits + i, res);
}

__global__ void k_naive(DeviceScene s, const float* __restrict__ rays, uint64_t n, gr_hit* __restrict__ hits) {
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + 6 * i;
    V3 o = V3{r[0], r[1], r[2]};
    V3 d = V3{r[3], r[4], r[5]};
    // Bvh::intersect_naive visits prims in order, then components; leaf order is a
    // permutation, so ties resolve by the lowest (prim, component) instead.
    TraceResult best{FLT_MAX, -1, 0.0f, 0.0f};
    uint64_t best_id = ~0ull;
    for (uint32_t k = 0; k < s.num_components; ++k) {
        const float4* pr = s.prims + 3 * static_cast<size_t>(k);
        float4 p0 = __ldg(pr), p1 = __ldg(pr + 1), p2 = __ldg(pr + 2);
        float u, v;
        float dist = intersect_prim(p0, p1, p2, o, d, u, v);
        if (dist == 0.0f) continue;
        uint64_t id = (static_cast<uint64_t>(__float_as_uint(p0.w)) << 32) | __float_as_uint(p1.w);
        if (dist < best.t || (dist == best.t && id < best_id)) {
            best = TraceResult{dist, static_cast<int32_t>(k), u, v};
            best_id = id;
        }
    }
    write_hit(s, hits + i, best);
}

template <int W>
__global__ void __launch_bounds__(QUERY_BLOCK) k_visibility(DeviceScene s, const float* __restrict__ pairs,
                                                            uint64_t n, uint8_t* __restrict__ vis, int* err) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pairs + 6 * i;
    V3 a = V3{p[0], p[1], p[2]};
    V3 b = V3{p[3], p[4], p[5]};
    // Bvh::visibility (geom/bvh.rs:460-477): a shadow ray from `a`, nudged, against
    // target distance - 1e-3; any hit closer than that occludes.
    if (fabsf(a.x - b.x) < 1e-3f && fabsf(a.y - b.y) < 1e-3f && fabsf(a.z - b.z) < 1e-3f) {
        vis[i] = 0;
        return;
    }
    V3 d = normalized(b - a);
    V3 o = nudge(a, d);
    float target = magnitude(b - o);
    TraceResult r = trace_ray<W, true>(s, o, d, target - 1e-3f, stk, err);
    vis[i] = r.k < 0 ? 1 : 0;
}

__global__ void k_sample_light(DeviceScene s, const float* __restrict__ u, uint64_t n, gr_light_sample* out) {
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float uu[6];
    for (int k = 0; k < 6; ++k) uu[k] = u[6 * i + k];
    DevLightSample ls = sample_light(s, uu);
    gr_light_sample o;
    auto put = [](float* d, V3 v) {
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
    };
    put(o.origin, ls.origin);
    put(o.direction, ls.direction);
    put(o.normal, ls.frame.normal);
    put(o.tangent, ls.frame.tangent);
    put(o.binormal, ls.frame.binormal);
    put(o.geom_normal, ls.frame.geom_normal);
    o.prim = static_cast<int32_t>(ls.prim);
    o.point_pdf = ls.point_pdf;
    o.dir_pdf = ls.dir_pdf;
    out[i] = o;
}

GR_D Frame frame_of(const gr_frame& f) {
    return Frame{V3{f.normal[0], f.normal[1], f.normal[2]}, V3{f.tangent[0], f.tangent[1], f.tangent[2]},
                 V3{f.binormal[0], f.binormal[1], f.binormal[2]},
                 V3{f.geom_normal[0], f.geom_normal[1], f.geom_normal[2]}};
}

__global__ void k_bsdf(int op, const DevMaterial* __restrict__ mp, uint64_t n, const gr_frame* __restrict__ frames,
                       const float* __restrict__ wi, const float* __restrict__ wo, const float* __restrict__ u,
                       int c2l, void* out) {
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevMaterial& m = *mp;
    Frame f = frame_of(frames[i]);
    V3 vi = V3{wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]};
    if (op == 0) {
        V3 vo = V3{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
        V3 r = f_world(m, vi, vo, f, c2l != 0);
        float* o = static_cast<float*>(out) + 3 * i;
        o[0] = r.x;
        o[1] = r.y;
        o[2] = r.z;
    } else if (op == 1) {
        V3 vo = V3{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
        static_cast<float*>(out)[i] = pdf_world(m, vi, vo, f);
    } else if (op == 2) {
        MaterialSample s = sample_world(m, vi, f, c2l != 0, u[3 * i], u[3 * i + 1], u[3 * i + 2]);
        gr_bsdf_sample o;
        o.emission[0] = s.emission.x;
        o.emission[1] = s.emission.y;
        o.emission[2] = s.emission.z;
        o.radiance[0] = s.radiance.x;
        o.radiance[1] = s.radiance.y;
        o.radiance[2] = s.radiance.z;
        o.outgoing[0] = s.outgoing.x;
        o.outgoing[1] = s.outgoing.y;
        o.outgoing[2] = s.outgoing.z;
        o.pdf = s.pdf;
        o.kind = s.kind;
        static_cast<gr_bsdf_sample*>(out)[i] = o;
    } else {
        V3 r = light_world(m, vi, f);
        float* o = static_cast<float*>(out) + 3 * i;
        o[0] = r.x;
        o[1] = r.y;
        o[2] = r.z;
    }
}

unsigned blocks_for(uint64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

template <int W>
gr_status trace_w(const DeviceScene& s, const float* rays, uint64_t n, gr_hit* hits, bool any, const float* tmax,
                  int* err, cudaStream_t st) {
    size_t smem = step_stack_smem_bytes(QUERY_BLOCK);
    if (any) {
        GR_CUDA_TRY(cudaFuncSetAttribute(k_trace<W, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
        k_trace<W, true><<<blocks_for(n, QUERY_BLOCK), QUERY_BLOCK, smem, st>>>(s, rays, n, hits, tmax, err);
    } else {
        GR_CUDA_TRY(cudaFuncSetAttribute(k_trace<W, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
        k_trace<W, false><<<blocks_for(n, QUERY_BLOCK), QUERY_BLOCK, smem, st>>>(s, rays, n, hits, tmax, err);
    }
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

template <int W>
gr_status vis_w(const DeviceScene& s, const float* pairs, uint64_t n, uint8_t* vis, int* err, cudaStream_t st) {
    size_t smem = step_stack_smem_bytes(QUERY_BLOCK);
    GR_CUDA_TRY(
        cudaFuncSetAttribute(k_visibility<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    k_visibility<W><<<blocks_for(n, QUERY_BLOCK), QUERY_BLOCK, smem, st>>>(s, pairs, n, vis, err);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

}  // namespace

gr_status launch_trace(const DeviceScene& s, const float* rays, uint64_t n, gr_hit* hits, bool any_hit,
                       const float* tmax, int* err, cudaStream_t st) {
    if (n == 0) return GR_OK;
    switch (s.width) {
        case 2: return trace_w<2>(s, rays, n, hits, any_hit, tmax, err, st);
        case 4: return trace_w<4>(s, rays, n, hits, any_hit, tmax, err, st);
        case 8: return trace_w<8>(s, rays, n, hits, any_hit, tmax, err, st);
    }
    set_error("unsupported BVH width");
    return GR_ERR_INTERNAL;
}

gr_status launch_naive(const DeviceScene& s, const float* rays, uint64_t n, gr_hit* hits, cudaStream_t st) {
    if (n == 0) return GR_OK;
    k_naive<<<blocks_for(n, 128), 128, 0, st>>>(s, rays, n, hits);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status launch_visibility(const DeviceScene& s, const float* pairs, uint64_t n, uint8_t* vis, int* err,
                            cudaStream_t st) {
    if (n == 0) return GR_OK;
    switch (s.width) {
        case 2: return vis_w<2>(s, pairs, n, vis, err, st);
        case 4: return vis_w<4>(s, pairs, n, vis, err, st);
        case 8: return vis_w<8>(s, pairs, n, vis, err, st);
    }
    set_error("unsupported BVH width");
    return GR_ERR_INTERNAL;
}

gr_status launch_sample_light(const DeviceScene& s, const float* u, uint64_t n, gr_light_sample* out,
                              cudaStream_t st) {
    if (n == 0) return GR_OK;
    k_sample_light<<<blocks_for(n, 128), 128, 0, st>>>(s, u, n, out);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

gr_status launch_bsdf(int op, const DevMaterial* m, uint64_t n, const gr_frame* frames, const float* wi,
                      const float* wo, const float* u, int c2l, void* out, cudaStream_t st) {
    if (n == 0) return GR_OK;
    k_bsdf<<<blocks_for(n, 128), 128, 0, st>>>(op, m, n, frames, wi, wo, u, c2l, out);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

}  // namespace gr
