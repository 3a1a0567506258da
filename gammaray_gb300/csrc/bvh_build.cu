// Device BVH build (GR_BUILD_DEVICE_LBVH): a linear BVH made on the GPU, then collapsed
// into the same wide node layout as the host build, so traversal is unchanged.
//
//   bounds     centroid bounds of all components (block reduction + ordered-int atomics)
//   morton     30-bit Morton code of each centroid in those bounds
//   sort       codes with component indices (CUB radix sort, stable: equal codes keep
//              component order)
//   tree       binary radix tree over the sorted codes (Karras, "Maximizing parallelism
//              in the construction of BVHs, octrees, and k-d trees", HPG 2012): internal
//              node i finds its key range and split from common-prefix lengths; equal
//              codes are told apart by their sorted index
//   boxes      bottom-up: each leaf walks to the root; the second child to arrive at a
//              node computes its box (counter atomics, no waiting)
//   collapse   level by level from the root: a wide node takes its binary node's two
//              children and opens the largest-area child holding more than `leaf_size`
//              components until it has `width` children; a child of at most `leaf_size`
//              components becomes one leaf over its contiguous range
//   stack      exact worst-case traversal stack use, deepest level first (as the host
//              collapse computes it)
//   records    primitive records and attribute indices permuted into leaf order
//
// The tree differs from the reference's SAH tree; closest hits do not (a ray keeps the
// nearest hit over all primitives), except that a tie at exactly equal distance may go
// to the other primitive.
#include <cfloat>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "runtime.hpp"
#include "traverse.cuh"  // MAX_STACK, the traversal stack bound

namespace gr {

namespace {

constexpr int BB = 256;  // threads per block of the build kernels

// Float <-> int that orders like the float, for atomicMin / atomicMax.
GR_D int ordered(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
GR_D float unordered(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

// Centroid = 0.5 lo + 0.5 hi (bvh.rs:26).
GR_D V3 centroid(const float* __restrict__ box, uint32_t k) {
    const float* b = box + 6 * static_cast<size_t>(k);
    return V3{0.5f * b[0] + 0.5f * b[3], 0.5f * b[1] + 0.5f * b[4], 0.5f * b[2] + 0.5f * b[5]};
}

__global__ void k_centroid_bounds(const float* __restrict__ box, uint32_t n, int* bounds) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        V3 c = centroid(box, k);
        float v[3] = {c.x, c.y, c.z};
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], v[a]);
            hi[a] = fmaxf(hi[a], v[a]);
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(bounds + a, ordered(lo[a]));
            atomicMax(bounds + 3 + a, ordered(hi[a]));
        }
}

// Spreads the low 10 bits of v to every third bit.
GR_D uint32_t spread3(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_morton(const float* __restrict__ box, uint32_t n, const int* __restrict__ bounds,
                         uint32_t* __restrict__ code, uint32_t* __restrict__ index) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    V3 c = centroid(box, k);
    float v[3] = {c.x, c.y, c.z};
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        float lo = unordered(bounds[a]), hi = unordered(bounds[3 + a]);
        float ext = hi - lo;
        float t = ext > 0.0f ? (v[a] - lo) / ext : 0.5f;
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        q[a] = min(1023u, static_cast<uint32_t>(t * 1024.0f));
    }
    code[k] = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
    index[k] = k;
}

// Common-prefix length of sorted keys i and j (codes, then sorted indices); -1 out of range.
GR_D int delta(const uint32_t* __restrict__ code, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = code[i], b = code[j];
    if (a == b) return 32 + __clz(static_cast<uint32_t>(i ^ j));
    return __clz(a ^ b);
}

// Child references: >= 0 an internal node, < 0 the leaf (sorted component) ~ref.
__global__ void k_radix_tree(const uint32_t* __restrict__ code, int n, int2* __restrict__ child,
                             int2* __restrict__ range, int* __restrict__ parent_internal,
                             int* __restrict__ parent_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = delta(code, n, i, i + 1) - delta(code, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = delta(code, n, i, i - d);
    int lmax = 2;
    while (delta(code, n, i, i + lmax * d) > dmin) lmax <<= 1;  // at most log2(n) + 1 doublings
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(code, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(code, n, i, j);
    int s = 0;
    for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
        if (delta(code, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = lo == gamma ? ~gamma : gamma;
    const int right = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(lo, hi);
    if (left >= 0) parent_internal[left] = i;
    else parent_leaf[~left] = i;
    if (right >= 0) parent_internal[right] = i;
    else parent_leaf[~right] = i;
}

struct NodeBox {
    float lo[3], hi[3];
};

GR_D NodeBox leaf_box(const float* __restrict__ box, const uint32_t* __restrict__ perm, int k) {
    const float* b = box + 6 * static_cast<size_t>(perm[k]);
    return NodeBox{{b[0], b[1], b[2]}, {b[3], b[4], b[5]}};
}

// Reads an internal node's box written by another thread (past L1).
GR_D NodeBox load_node_box(const NodeBox* nb, int i) {
    const float* f = reinterpret_cast<const float*>(nb + i);
    NodeBox r;
    for (int a = 0; a < 3; ++a) {
        r.lo[a] = __ldcg(f + a);
        r.hi[a] = __ldcg(f + 3 + a);
    }
    return r;
}

__global__ void k_boxes(const float* __restrict__ box, const uint32_t* __restrict__ perm, int n,
                        const int2* __restrict__ child, const int* __restrict__ parent_internal,
                        const int* __restrict__ parent_leaf, NodeBox* node_box, int* visits, int* err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int p = parent_leaf[k];
    for (int steps = 0; p >= 0; ++steps) {
        if (steps >= n) {  // a parent chain longer than the tree: flag it, never loop
            atomicExch(err, 1);
            return;
        }
        __threadfence();  // this child's box is visible before the count
        if (atomicAdd(visits + p, 1) == 0) return;  // the sibling will finish the node
        int2 c = child[p];
        NodeBox a = c.x < 0 ? leaf_box(box, perm, ~c.x) : load_node_box(node_box, c.x);
        NodeBox b = c.y < 0 ? leaf_box(box, perm, ~c.y) : load_node_box(node_box, c.y);
        NodeBox u;
        for (int q = 0; q < 3; ++q) {
            u.lo[q] = fminf(a.lo[q], b.lo[q]);
            u.hi[q] = fmaxf(a.hi[q], b.hi[q]);
        }
        node_box[p] = u;
        p = parent_internal[p];
    }
}

struct Cand {
    int ref;  // binary node (>= 0) or leaf ~k
    int first, count;
};

GR_D Cand cand_of(int ref, const int2* __restrict__ range) {
    if (ref < 0) return Cand{ref, ~ref, 1};
    int2 r = range[ref];
    return Cand{ref, r.x, r.y - r.x + 1};
}

GR_D NodeBox cand_box(const Cand& c, const float* __restrict__ box, const uint32_t* __restrict__ perm,
                      const NodeBox* __restrict__ node_box) {
    return c.ref < 0 ? leaf_box(box, perm, ~c.ref) : node_box[c.ref];
}

GR_D float half_area(const NodeBox& b) {
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

struct CollapseOut {
    float* nodes;        // 8 * W floats per wide node
    int2* next;          // (wide node, binary ref) of the next level
    uint32_t* next_n;
    uint32_t* wide_n;
    uint32_t* nchild;    // per wide node: its slots in use
};

// One wide node per frontier entry (wide index, binary node it stands for).
template <int W>
__global__ void k_collapse(const int2* __restrict__ frontier, uint32_t n_front, const int2* __restrict__ child,
                           const int2* __restrict__ range, const float* __restrict__ box,
                           const uint32_t* __restrict__ perm, const NodeBox* __restrict__ node_box,
                           uint32_t leaf_size, CollapseOut o) {
    uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_front) return;
    const int wide = frontier[f].x, bin = frontier[f].y;
    Cand c[W];
    int nc = 0;
    Cand root = cand_of(bin, range);
    if (bin >= 0 && root.count > static_cast<int>(leaf_size)) {
        int2 ch = child[bin];
        c[nc++] = cand_of(ch.x, range);
        c[nc++] = cand_of(ch.y, range);
    } else {
        c[nc++] = root;
    }
    while (nc < W) {  // open the largest-area child that is still too big for a leaf
        int best = -1;
        float best_area = -1.0f;
        for (int q = 0; q < nc; ++q) {
            if (c[q].ref < 0 || c[q].count <= static_cast<int>(leaf_size)) continue;
            float a = half_area(node_box[c[q].ref]);
            if (!(a <= best_area)) {
                best = q;
                best_area = a;
            }
        }
        if (best < 0) break;
        int2 ch = child[c[best].ref];
        for (int q = nc; q > best + 1; --q) c[q] = c[q - 1];
        c[best] = cand_of(ch.x, range);
        c[best + 1] = cand_of(ch.y, range);
        ++nc;
    }
    float* node = o.nodes + static_cast<size_t>(wide) * 8 * W;
    for (int j = 0; j < W; ++j) {
        NodeBox b{{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}};  // empty slots never hit
        int ref = ~0;
        if (j < nc) {
            b = cand_box(c[j], box, perm, node_box);
            if (c[j].count <= static_cast<int>(leaf_size)) {
                ref = ~static_cast<int>((static_cast<uint32_t>(c[j].first) << LEAF_COUNT_BITS) |
                                        static_cast<uint32_t>(c[j].count - 1));
            } else {
                ref = static_cast<int>(atomicAdd(o.wide_n, 1u));
                o.next[atomicAdd(o.next_n, 1u)] = make_int2(ref, c[j].ref);
            }
        }
        for (int a = 0; a < 3; ++a) {
            node[a * W + j] = b.lo[a];
            node[(3 + a) * W + j] = b.hi[a];
        }
        node[6 * W + j] = __int_as_float(ref);
    }
    for (int j = 6 * W + W; j < 8 * W; ++j) node[j] = 0.0f;
    o.nchild[wide] = static_cast<uint32_t>(nc);
}

// Worst-case stack use of a wide node's subtree: (children - 1) + the largest of its
// interior children's (host collapse: Collapser::emit).
template <int W>
__global__ void k_stack_use(const int2* __restrict__ level, uint32_t n, const float* __restrict__ nodes,
                            const uint32_t* __restrict__ nchild, uint32_t* su) {
    uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    const int wide = level[f].x;
    const float* node = nodes + static_cast<size_t>(wide) * 8 * W;
    uint32_t m = 0;
    for (int j = 0; j < W; ++j) {
        int ref = __float_as_int(node[6 * W + j]);
        if (j < static_cast<int>(nchild[wide]) && ref >= 0) m = max(m, su[ref]);
    }
    su[wide] = nchild[wide] - 1 + m;
}

__global__ void k_permute(const float4* __restrict__ rec, const uint32_t* __restrict__ tn,
                          const uint32_t* __restrict__ tu, const uint32_t* __restrict__ perm, uint32_t n,
                          float4* __restrict__ rec_out, uint32_t* __restrict__ tn_out, uint32_t* __restrict__ tu_out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t s = perm[k];
    for (int q = 0; q < 3; ++q) rec_out[3 * static_cast<size_t>(k) + q] = rec[3 * static_cast<size_t>(s) + q];
    if (tn)
        for (int q = 0; q < 3; ++q) tn_out[3 * static_cast<size_t>(k) + q] = tn[3 * static_cast<size_t>(s) + q];
    if (tu)
        for (int q = 0; q < 3; ++q) tu_out[3 * static_cast<size_t>(k) + q] = tu[3 * static_cast<size_t>(s) + q];
}

template <class T>
cudaError_t put(DevBuf& b, const T& v, cudaStream_t st) {
    cudaError_t e = b.ensure(v.size() * sizeof(v[0]));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice, st);
}

template <int W>
gr_status collapse_levels(uint32_t n, const int2* child, const int2* range, const float* box, const uint32_t* perm,
                          const NodeBox* node_box, uint32_t leaf_size, SceneBuffers& b, cudaStream_t st,
                          uint32_t& num_wide, uint32_t& stack_depth) {
    // Every wide node stands for a distinct binary node (or the root leaf): at most n.
    const size_t max_wide = std::max<size_t>(1, n);
    GR_CUDA_TRY(b.nodes.ensure(max_wide * 8 * W * sizeof(float)));
    DevBuf levels, ctr, nchild, su;
    GR_CUDA_TRY(levels.ensure(max_wide * sizeof(int2)));
    GR_CUDA_TRY(ctr.ensure(2 * sizeof(uint32_t)));
    GR_CUDA_TRY(nchild.ensure(max_wide * sizeof(uint32_t)));
    GR_CUDA_TRY(su.ensure(max_wide * sizeof(uint32_t)));
    int2 root = make_int2(0, n > 1 ? 0 : ~0);
    uint32_t init[2] = {1, 0};  // wide nodes, entries of the next level
    GR_CUDA_TRY(cudaMemcpyAsync(levels.ptr, &root, sizeof(int2), cudaMemcpyHostToDevice, st));
    GR_CUDA_TRY(cudaMemcpyAsync(ctr.ptr, init, sizeof(init), cudaMemcpyHostToDevice, st));
    // Levels are stored back to back in `levels`: [off[d], off[d] + len[d]).
    std::vector<uint32_t> off{0}, len{1};
    uint32_t* c = ctr.as<uint32_t>();
    for (uint32_t depth = 0; len.back() > 0; ++depth) {
        if (depth > n) {
            set_error("device BVH build: collapse did not terminate");
            return GR_ERR_INTERNAL;
        }
        const uint32_t nf = len.back(), start = off.back();
        GR_CUDA_TRY(cudaMemsetAsync(c + 1, 0, sizeof(uint32_t), st));
        CollapseOut o{b.nodes.as<float>(), levels.as<int2>() + start + nf, c + 1, c, nchild.as<uint32_t>()};
        k_collapse<W><<<(nf + BB - 1) / BB, BB, 0, st>>>(levels.as<int2>() + start, nf, child, range, box, perm,
                                                         node_box, leaf_size, o);
        GR_CUDA_TRY(cudaGetLastError());
        uint32_t next = 0;
        GR_CUDA_TRY(cudaMemcpyAsync(&next, c + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        GR_CUDA_TRY(cudaStreamSynchronize(st));
        off.push_back(start + nf);
        len.push_back(next);
    }
    GR_CUDA_TRY(cudaMemcpyAsync(&num_wide, c, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    for (size_t d = len.size() - 1; d-- > 0;) {  // deepest level first
        k_stack_use<W><<<(len[d] + BB - 1) / BB, BB, 0, st>>>(levels.as<int2>() + off[d], len[d], b.nodes.as<float>(),
                                                              nchild.as<uint32_t>(), su.as<uint32_t>());
        GR_CUDA_TRY(cudaGetLastError());
    }
    uint32_t root_su = 0;
    GR_CUDA_TRY(cudaMemcpyAsync(&root_su, su.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    stack_depth = root_su + 1;
    return GR_OK;
}

}  // namespace

gr_status build_bvh_device(const HostBuild& h, SceneBuffers& b, cudaStream_t st, uint32_t& num_wide,
                           uint32_t& stack_depth, uint64_t& bytes) {
    const uint32_t n = static_cast<uint32_t>(h.num_components);
    const uint32_t W = h.width, L = h.leaf_size;
    DevBuf box, rec, tn, tu, bounds, code, index, code_s, perm, child, range, par_i, par_l, nbox, visits, err, tmp;
    GR_CUDA_TRY(put(box, h.item_boxes, st));
    GR_CUDA_TRY(put(rec, h.prims, st));
    GR_CUDA_TRY(put(tn, h.tri_normal_idx, st));
    GR_CUDA_TRY(put(tu, h.tri_uv_idx, st));
    int init[6];
    for (int a = 0; a < 3; ++a) {
        init[a] = 0x7FFFFFFF;  // ordered(+max)
        init[3 + a] = static_cast<int>(0x80000000u);
    }
    GR_CUDA_TRY(bounds.ensure(sizeof(init)));
    GR_CUDA_TRY(cudaMemcpyAsync(bounds.ptr, init, sizeof(init), cudaMemcpyHostToDevice, st));
    const uint32_t blocks = (n + BB - 1) / BB;
    k_centroid_bounds<<<std::min(blocks, 1024u), BB, 0, st>>>(box.as<float>(), n, bounds.as<int>());
    GR_CUDA_TRY(cudaGetLastError());
    GR_CUDA_TRY(code.ensure(n * sizeof(uint32_t)));
    GR_CUDA_TRY(index.ensure(n * sizeof(uint32_t)));
    GR_CUDA_TRY(code_s.ensure(n * sizeof(uint32_t)));
    GR_CUDA_TRY(perm.ensure(n * sizeof(uint32_t)));
    k_morton<<<blocks, BB, 0, st>>>(box.as<float>(), n, bounds.as<int>(), code.as<uint32_t>(), index.as<uint32_t>());
    GR_CUDA_TRY(cudaGetLastError());
    size_t tmp_bytes = 0;
    GR_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, code.as<uint32_t>(), code_s.as<uint32_t>(),
                                                index.as<uint32_t>(), perm.as<uint32_t>(), static_cast<int>(n), 0, 30,
                                                st));
    GR_CUDA_TRY(tmp.ensure(std::max<size_t>(tmp_bytes, 16)));
    GR_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp.ptr, tmp_bytes, code.as<uint32_t>(), code_s.as<uint32_t>(),
                                                index.as<uint32_t>(), perm.as<uint32_t>(), static_cast<int>(n), 0, 30,
                                                st));
    const uint32_t ni = n > 1 ? n - 1 : 1;  // internal nodes
    GR_CUDA_TRY(child.ensure(ni * sizeof(int2)));
    GR_CUDA_TRY(range.ensure(ni * sizeof(int2)));
    GR_CUDA_TRY(par_i.ensure(ni * sizeof(int)));
    GR_CUDA_TRY(par_l.ensure(n * sizeof(int)));
    GR_CUDA_TRY(nbox.ensure(ni * sizeof(NodeBox)));
    GR_CUDA_TRY(visits.ensure(ni * sizeof(int)));
    GR_CUDA_TRY(err.ensure(sizeof(int)));
    GR_CUDA_TRY(cudaMemsetAsync(par_i.ptr, 0xFF, ni * sizeof(int), st));  // root: -1
    GR_CUDA_TRY(cudaMemsetAsync(par_l.ptr, 0xFF, n * sizeof(int), st));
    GR_CUDA_TRY(cudaMemsetAsync(visits.ptr, 0, ni * sizeof(int), st));
    GR_CUDA_TRY(cudaMemsetAsync(err.ptr, 0, sizeof(int), st));
    if (n > 1) {
        k_radix_tree<<<(n - 1 + BB - 1) / BB, BB, 0, st>>>(code_s.as<uint32_t>(), static_cast<int>(n), child.as<int2>(),
                                                           range.as<int2>(), par_i.as<int>(), par_l.as<int>());
        GR_CUDA_TRY(cudaGetLastError());
        k_boxes<<<blocks, BB, 0, st>>>(box.as<float>(), perm.as<uint32_t>(), static_cast<int>(n), child.as<int2>(),
                                       par_i.as<int>(), par_l.as<int>(), nbox.as<NodeBox>(), visits.as<int>(),
                                       err.as<int>());
        GR_CUDA_TRY(cudaGetLastError());
    }
    int e = 0;
    GR_CUDA_TRY(cudaMemcpyAsync(&e, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    if (e) {
        set_error("device BVH build: inconsistent radix tree");
        return GR_ERR_INTERNAL;
    }
    gr_status s;
    switch (W) {
        case 2: s = collapse_levels<2>(n, child.as<int2>(), range.as<int2>(), box.as<float>(), perm.as<uint32_t>(),
                                       nbox.as<NodeBox>(), L, b, st, num_wide, stack_depth); break;
        case 8: s = collapse_levels<8>(n, child.as<int2>(), range.as<int2>(), box.as<float>(), perm.as<uint32_t>(),
                                       nbox.as<NodeBox>(), L, b, st, num_wide, stack_depth); break;
        default: s = collapse_levels<4>(n, child.as<int2>(), range.as<int2>(), box.as<float>(), perm.as<uint32_t>(),
                                        nbox.as<NodeBox>(), L, b, st, num_wide, stack_depth); break;
    }
    if (s != GR_OK) return s;
    if (stack_depth > static_cast<uint32_t>(MAX_STACK)) {
        set_error("device BVH build: the tree needs a traversal stack of " + std::to_string(stack_depth) +
                  " entries (limit " + std::to_string(MAX_STACK) + ")");
        return GR_ERR_STACK_OVERFLOW;
    }
    GR_CUDA_TRY(b.prims.ensure(h.prims.size() * sizeof(float)));
    GR_CUDA_TRY(b.tri_nidx.ensure(h.tri_normal_idx.size() * sizeof(uint32_t)));
    GR_CUDA_TRY(b.tri_uvidx.ensure(h.tri_uv_idx.size() * sizeof(uint32_t)));
    k_permute<<<blocks, BB, 0, st>>>(rec.as<float4>(), h.tri_normal_idx.empty() ? nullptr : tn.as<uint32_t>(),
                                     h.tri_uv_idx.empty() ? nullptr : tu.as<uint32_t>(), perm.as<uint32_t>(), n,
                                     b.prims.as<float4>(), b.tri_nidx.as<uint32_t>(), b.tri_uvidx.as<uint32_t>());
    GR_CUDA_TRY(cudaGetLastError());
    GR_CUDA_TRY(cudaStreamSynchronize(st));
    bytes += static_cast<uint64_t>(num_wide) * 8 * W * sizeof(float) + h.prims.size() * sizeof(float) +
             (h.tri_normal_idx.size() + h.tri_uv_idx.size()) * sizeof(uint32_t);
    return GR_OK;
}

}  // namespace gr
