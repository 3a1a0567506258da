// Host-side scene build: materials, the reference SAH BVH, and its collapse into the
// device's wide layout.
//
// The binary build follows geom/bvh.rs:182-382 step by step, including its quirks
// (they change the tree, never which triangle a ray hits):
//   - BBox::surface_area returns the volume (core/bbox.rs:73-76), so flat nodes give
//     NaN costs and fall through to a median split;
//   - the SAH "leaf" branch still median-splits (bvh.rs:290-296), so leaves hold one
//     component unless centroids coincide;
//   - nth_element's left recursion range stops one short of the pivot (geom/util.rs:40);
//   - maximum_extent picks x only when y >= z as well (core/bbox.rs:44-56).
// The binary tree is then collapsed into nodes of `width` children: a child whose
// subtree holds at most `leaf_size` components becomes one leaf over its contiguous
// component range; otherwise the interior child of largest surface area is opened
// until the node is full.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <numeric>
#include <pthread.h>
#include <unistd.h>
#include <condition_variable>
#include <mutex>
#include <thread>

#include "scene.hpp"

namespace gr {

namespace {

struct Box {
    float lo[3], hi[3];
    static Box empty() {
        Box b;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = FLT_MAX;
            b.hi[k] = -FLT_MAX;
        }
        return b;
    }
    void grow(const Box& o) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], o.lo[k]);
            hi[k] = fmaxf(hi[k], o.hi[k]);
        }
    }
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], p[k]);
            hi[k] = fmaxf(hi[k], p[k]);
        }
    }
    float volume() const { return (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]); }
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
    int max_extent() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx >= dy && dy >= dz) return 0;
        if (dy >= dz) return 1;
        return 2;
    }
};

struct Item {
    uint32_t prim, comp;
    Box box;
    float cen[3];
};

struct BinNode {
    Box box;
    int32_t child[2];  // -1 for leaves
    uint32_t first, count;  // component range of the whole subtree
};
// Arrays written in full after they are sized: no zero fill.
using BinNodes = std::vector<BinNode, NoInitAlloc<BinNode>>;

// One component during the binary build: its box, centroid and item index.  The build
// permutes these records in place (not an index array into the items), so each pass
// over a node's range reads memory in order.  The high bits of `id` carry the SAH
// bucket between the bucket count and the partition of the same node.
struct Rec {
    Box box;
    float cen[3];
    uint32_t id;
};
// A thread with a large stack: the reference's build recurses once per tree level, and
// a skewed split (one component against the rest) adds a level per component.  64 MB
// holds about 70,000 levels; the memory is committed only as it is touched.
class BuildThread {
  public:
    static constexpr size_t STACK = size_t(64) << 20;
    explicit BuildThread(std::function<void()> fn) : fn_(std::move(fn)) {
        pthread_attr_t at;
        pthread_attr_init(&at);
        pthread_attr_setstacksize(&at, STACK);
        ok_ = pthread_create(&t_, &at, &BuildThread::entry, this) == 0;
        pthread_attr_destroy(&at);
        if (!ok_) fn_();  // no thread: run here
    }
    void join() {
        if (ok_) pthread_join(t_, nullptr);
        ok_ = false;
    }
    ~BuildThread() { join(); }

  private:
    static void* entry(void* self) {
        static_cast<BuildThread*>(self)->fn_();
        return nullptr;
    }
    std::function<void()> fn_;
    pthread_t t_{};
    bool ok_ = false;
};

// Worker threads for the build's data-parallel passes, started on first use and kept
// for the life of the process (heap-allocated and detached: no destructor runs while a
// worker waits).  run() splits a pass into parts taken by the workers and the calling
// thread, so it completes even with no worker free; in a forked child (no workers) the
// caller runs every part itself.
class PassPool {
  public:
    static PassPool& get() {
        static PassPool* pool = new PassPool();
        return *pool;
    }
    void run(unsigned parts, const std::function<void(unsigned)>& fn) {
        if (parts <= 1 || getpid() != pid_ || workers_ == 0) {
            for (unsigned k = 0; k < parts; ++k) fn(k);
            return;
        }
        Job job;
        job.fn = &fn;
        job.parts = parts;
        {
            std::lock_guard<std::mutex> g(mu_);
            jobs_.push_back(&job);
            open_.fetch_add(1);
        }
        cv_.notify_all();
        work(job);
        {
            std::lock_guard<std::mutex> g(mu_);
            for (size_t i = 0; i < jobs_.size(); ++i)
                if (jobs_[i] == &job) {
                    jobs_.erase(jobs_.begin() + static_cast<long>(i));
                    break;
                }
        }
        while (job.done.load() != parts || job.inside.load() != 0) std::this_thread::yield();
    }

  private:
    struct Job {
        const std::function<void(unsigned)>* fn = nullptr;
        unsigned parts = 0;
        std::atomic<unsigned> next{0}, done{0}, inside{0};
    };
    // Runs parts of j until none is left; the thread that first finds none closes it.
    void work(Job& j) {
        for (;;) {
            unsigned k = j.next.fetch_add(1);
            if (k >= j.parts) {
                if (k == j.parts) open_.fetch_sub(1);
                return;
            }
            (*j.fn)(k);
            j.done.fetch_add(1);
        }
    }
    PassPool() : pid_(getpid()) {
        unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        workers_ = hw - 1;
        for (unsigned i = 0; i < workers_; ++i) std::thread([this] { loop(); }).detach();
    }
    // Takes a part of the first job that has parts left; spins a little before sleeping,
    // as a build's passes follow one another closely.
    void loop() {
        for (;;) {
            Job* j = nullptr;
            for (int spin = 0; spin < 2000 && !j; ++spin) {
                if (open_.load() != 0) j = take();
                if (!j) std::this_thread::yield();
            }
            if (!j) {
                std::unique_lock<std::mutex> l(mu_);
                cv_.wait(l, [&] { return open_.load() != 0; });
                l.unlock();
                j = take();
            }
            if (j) {
                work(*j);
                j->inside.fetch_sub(1);  // the caller may return from run() after this
            }
        }
    }
    Job* take() {
        std::lock_guard<std::mutex> g(mu_);
        for (Job* j : jobs_)
            if (j->next.load() < j->parts) {
                j->inside.fetch_add(1);
                return j;
            }
        return nullptr;
    }
    std::mutex mu_;
    std::condition_variable cv_;
    std::vector<Job*> jobs_;
    std::atomic<int> open_{0};  // jobs with parts not yet taken
    unsigned workers_ = 0;
    pid_t pid_;
};

constexpr int ID_BITS = 31 - LEAF_COUNT_BITS;  // components < 2^ID_BITS (checked before the build)
constexpr uint32_t ID_MASK = (1u << ID_BITS) - 1u;

// The reference's recursive build (geom/bvh.rs:182-382).  Every choice depends only on
// the records of the node's range and their order, so subtrees are built on separate
// threads with the same result.  Node numbering is free (the collapse follows child
// links): each thread takes nodes from its own chunks of CHUNK slots, so a subtree's
// nodes sit together.  A leaf's first component is its offset in the record array, which
// is the reference's leaf order.
class RefBuilder {
  public:
    static constexpr size_t SPAWN_MIN = 2048;    // smaller subtrees stay on their thread
    static constexpr size_t SPLIT_PASS = 32768;  // larger nodes split their passes
    static constexpr uint32_t CHUNK = 1024;      // node slots taken at a time by a thread

    // A thread's current chunk of node slots.
    struct Alloc {
        uint32_t next = 0, end = 0, used = 0;
    };

    Rec* base;
    std::unique_ptr<Rec[]> tmp;  // scratch for the parallel partition (same indexing as base)
    BinNodes nodes;
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> used{0};
    unsigned threads = 1;
    int spawn_depth = 0;

    RefBuilder(Rec* recs, size_t n) : base(recs) {
        threads = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        // SAH splits are uneven: spawn about four subtrees per thread.
        while (spawn_depth < 8 && (1u << spawn_depth) < 4 * threads) ++spawn_depth;
        if (threads == 1 || n < 2 * SPAWN_MIN) spawn_depth = 0;
        // At most 2n - 1 nodes, plus the unused tail of each thread's last chunk.
        nodes.resize(2 * n + (static_cast<size_t>(2) << spawn_depth) * CHUNK);
        if (threads > 1 && n >= SPLIT_PASS) tmp.reset(new Rec[n]);
    }

    // The reference's swap partition computed on the pass pool, with the same result:
    // the matches keep their order at the front; the others behave like a queue that
    // moves its front element to its back at every later match.  So with p1 the first
    // non-match, T the indices of the matches after it and R = |T|, the non-match at
    // index p ends at k + pos - R, where pos starts at p - p1 and steps pos = T[pos] - p1
    // while pos < R (k: the number of matches).
    template <class P>
    size_t partition_parallel(Rec* s, size_t n, const P& pred) {
        const unsigned parts = threads;
        std::vector<size_t> before(parts + 1, 0);  // matches before each part
        in_parts(n, parts, [&](unsigned k, size_t b, size_t e) {
            size_t c = 0;
            for (size_t i = b; i < e; ++i) c += pred(s[i]) ? 1 : 0;
            before[k + 1] = c;
        });
        for (unsigned k = 0; k < parts; ++k) before[k + 1] += before[k];
        const size_t k_all = before[parts];
        if (k_all == n || k_all == 0) return k_all;  // nothing moves
        size_t p1 = 0;
        while (pred(s[p1])) ++p1;  // the first non-match (all before it match)
        const size_t R = k_all - p1;
        std::vector<uint32_t> T(R);
        Rec* out = tmp.get() + (s - base);
        in_parts(n, parts, [&](unsigned k, size_t b, size_t e) {
            size_t q = before[k];  // rank of the next match
            for (size_t i = b; i < e; ++i)
                if (pred(s[i])) {
                    if (i > p1) T[q - p1] = static_cast<uint32_t>(i);
                    out[q++] = s[i];
                }
        });
        in_parts(n, parts, [&](unsigned, size_t b, size_t e) {
            for (size_t i = b; i < e; ++i)
                if (!pred(s[i])) {
                    size_t pos = i - p1;
                    while (pos < R) pos = T[pos] - p1;
                    out[k_all + pos - R] = s[i];
                }
        });
        in_parts(n, parts, [&](unsigned, size_t b, size_t e) { std::memcpy(s + b, out + b, (e - b) * sizeof(Rec)); });
        return k_all;
    }

    uint64_t node_count() const { return used.load(); }

    // Runs fn(k, begin, end) over `parts` contiguous pieces of [0, n), on the pass pool.
    template <class F>
    static void in_parts(size_t n, unsigned parts, const F& fn) {
        PassPool::get().run(parts, [&](unsigned k) { fn(k, n * k / parts, n * (k + 1) / parts); });
    }

    static int bucket(const Box& cb, const float* c, int dim) {
        const int NB = 12;
        float rel = (c[dim] - cb.lo[dim]) / (cb.hi[dim] - cb.lo[dim]);
        float f = static_cast<float>(NB) * rel;
        long long b = (f >= 0.0f) ? static_cast<long long>(f) : 0;  // `as usize` saturates at 0
        if (b > NB - 1) b = NB - 1;
        return static_cast<int>(b);
    }

    // The reference's unstable partition (geom/util.rs): swaps matches to the front.
    template <class P>
    static size_t partition(Rec* s, size_t len, const P& pred) {
        size_t cursor = 0;
        for (size_t i = 0; i < len; ++i)
            if (pred(s[i])) std::swap(s[i], s[cursor++]);
        return cursor;
    }

    static void nth_element(Rec* s, size_t len, size_t nth, int dim) {
        while (len >= 2) {
            size_t pivot = len / 2;
            std::swap(s[pivot], s[len - 1]);
            float pv = s[len - 1].cen[dim];
            size_t fpi = partition(s, len - 1, [&](const Rec& x) { return x.cen[dim] < pv; });
            std::swap(s[len - 1], s[fpi]);
            if (nth < fpi) {
                len = fpi - 1;  // one short of the pivot, as geom/util.rs:40
            } else if (nth > fpi) {
                s += fpi + 1;
                len -= fpi + 1;
                nth -= fpi + 1;
            } else {
                return;
            }
        }
    }

    // Node box and centroid box.  min / max are exact, so a split pass gives the
    // serial result.
    void bounds(const Rec* s, size_t n, Box& box, Box& cb) const {
        box = Box::empty();
        cb = Box::empty();
        if (n < SPLIT_PASS || threads == 1) {
            for (size_t i = 0; i < n; ++i) {
                box.grow(s[i].box);
                cb.grow(s[i].cen);
            }
            return;
        }
        std::vector<Box> pb(threads, Box::empty()), pc(threads, Box::empty());
        in_parts(n, threads, [&](unsigned k, size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) {
                pb[k].grow(s[i].box);
                pc[k].grow(s[i].cen);
            }
        });
        for (unsigned k = 0; k < threads; ++k) {
            box.grow(pb[k]);
            cb.grow(pc[k]);
        }
    }

    // SAH bucket of each record (kept in its id's high bits), with per-bucket counts,
    // boxes and centroid bounds (from which the children's bounds follow exactly).
    template <int NB>
    void buckets(Rec* s, size_t n, const Box& cb, int dim, size_t* count, Box* bb, Box* cbb) const {
        auto pass = [&](size_t b, size_t e, size_t* c, Box* x, Box* y) {
            for (size_t i = b; i < e; ++i) {
                int k = bucket(cb, s[i].cen, dim);
                s[i].id = (s[i].id & ID_MASK) | (static_cast<uint32_t>(k) << ID_BITS);
                c[k] += 1;
                x[k].grow(s[i].box);
                y[k].grow(s[i].cen);
            }
        };
        for (int b = 0; b < NB; ++b) {
            count[b] = 0;
            bb[b] = Box::empty();
            cbb[b] = Box::empty();
        }
        if (n < SPLIT_PASS || threads == 1) {
            pass(0, n, count, bb, cbb);
            return;
        }
        std::vector<size_t> pc(threads * NB, 0);
        std::vector<Box> px(threads * NB, Box::empty()), py(threads * NB, Box::empty());
        in_parts(n, threads,
                 [&](unsigned k, size_t b, size_t e) { pass(b, e, &pc[k * NB], &px[k * NB], &py[k * NB]); });
        for (unsigned k = 0; k < threads; ++k)
            for (int b = 0; b < NB; ++b) {
                count[b] += pc[k * NB + b];
                bb[b].grow(px[k * NB + b]);
                cbb[b].grow(py[k * NB + b]);
            }
    }

    int32_t build(Rec* s, size_t n) {
        int32_t root = -1;
        BuildThread t([&] {
            Alloc a;
            root = build(s, n, 0, a, nullptr);
            used += a.used;
        });
        t.join();
        return root;
    }

    // `known`, when given, holds the range's box and centroid box.
    int32_t build(Rec* s, size_t n, int depth, Alloc& a, const Box* known) {
        Box box, cb;
        if (known) {
            box = known[0];
            cb = known[1];
        } else {
            bounds(s, n, box, cb);
        }
        if (n == 1) return leaf(s, n, box, a);
        int dim = cb.max_extent();
        if (cb.lo[dim] == cb.hi[dim]) return leaf(s, n, box, a);
        size_t mid;
        Box kids[4] = {Box::empty(), Box::empty(), Box::empty(), Box::empty()};  // box, centroid box per side
        bool kids_known = false;
        if (n <= 4) {
            mid = n / 2;
            nth_element(s, n, mid, dim);
        } else {
            constexpr int NB = 12;
            size_t count[NB];
            Box bb[NB], cbb[NB];
            buckets<NB>(s, n, cb, dim, count, bb, cbb);
            float cost[NB - 1];
            for (int i = 0; i < NB - 1; ++i) {
                Box b0 = Box::empty(), b1 = Box::empty();
                size_t c0 = 0, c1 = 0;
                for (int j = 0; j <= i; ++j) {
                    b0.grow(bb[j]);
                    c0 += count[j];
                }
                for (int j = i + 1; j < NB; ++j) {
                    b1.grow(bb[j]);
                    c1 += count[j];
                }
                cost[i] = 1.0f + (static_cast<float>(c0) * b0.volume() + static_cast<float>(c1) * b1.volume()) /
                                     box.volume();
            }
            float min_cost = cost[0];
            int min_b = 0;
            for (int i = 1; i < NB - 1; ++i)
                if (cost[i] < min_cost) {
                    min_cost = cost[i];
                    min_b = i;
                }
            if (n > 255 || min_cost < static_cast<float>(n)) {
                const uint32_t mb = static_cast<uint32_t>(min_b);
                auto left = [&](const Rec& x) { return (x.id >> ID_BITS) <= mb; };
                mid = (n >= SPLIT_PASS && tmp) ? partition_parallel(s, n, left) : partition(s, n, left);
                for (int b = 0; b < NB; ++b) {
                    Box* side = b <= min_b ? kids : kids + 2;
                    side[0].grow(bb[b]);
                    side[1].grow(cbb[b]);
                }
                kids_known = true;
            } else {
                mid = n / 2;
                nth_element(s, n, mid, dim);
            }
        }
        const Box* k0 = kids_known ? kids : nullptr;
        const Box* k1 = kids_known ? kids + 2 : nullptr;
        int32_t c0, c1;
        if (depth < spawn_depth && mid >= SPAWN_MIN && n - mid >= SPAWN_MIN) {
            BuildThread left([&] {
                Alloc la;
                c0 = build(s, mid, depth + 1, la, k0);
                used += la.used;
            });
            c1 = build(s + mid, n - mid, depth + 1, a, k1);
            left.join();
        } else {
            c0 = build(s, mid, depth + 1, a, k0);
            c1 = build(s + mid, n - mid, depth + 1, a, k1);
        }
        BinNode nd;
        nd.box = nodes[c0].box;
        nd.box.grow(nodes[c1].box);
        nd.child[0] = c0;
        nd.child[1] = c1;
        nd.first = nodes[c0].first;
        nd.count = nodes[c0].count + nodes[c1].count;
        return put(nd, a);
    }

    int32_t leaf(Rec* s, size_t n, const Box& box, Alloc& a) {
        BinNode nd;
        nd.box = box;
        nd.child[0] = nd.child[1] = -1;
        nd.first = static_cast<uint32_t>(s - base);
        nd.count = static_cast<uint32_t>(n);
        return put(nd, a);
    }

    int32_t put(const BinNode& nd, Alloc& a) {
        if (a.next == a.end) {
            a.next = next.fetch_add(CHUNK, std::memory_order_relaxed);
            a.end = a.next + CHUNK;
        }
        nodes[a.next] = nd;
        ++a.used;
        return static_cast<int32_t>(a.next++);
    }
};

// A slot candidate during the collapse: a binary node, or a plain component range
// (used to split oversized binary leaves).
struct Cand {
    int32_t bin;  // -1 for a range
    uint32_t first, count;
    Box box;
};

class Collapser {
  public:
    const BinNodes& bin;
    const std::vector<Box, NoInitAlloc<Box>>& comp_box;  // per ordered component
    uint32_t W, L;
    std::vector<float>& out;  // node floats

    Collapser(const BinNodes& b, const std::vector<Box, NoInitAlloc<Box>>& cb, uint32_t w, uint32_t l,
              std::vector<float>& o)
        : bin(b), comp_box(cb), W(w), L(l), out(o) {}

    Cand of_bin(int32_t b) const { return Cand{b, bin[b].first, bin[b].count, bin[b].box}; }
    Cand of_range(uint32_t first, uint32_t count) const {
        Box b = Box::empty();
        for (uint32_t i = first; i < first + count; ++i) b.grow(comp_box[i]);
        return Cand{-1, first, count, b};
    }
    bool expandable(const Cand& c) const { return c.count > L; }
    void expand(const Cand& c, Cand& a, Cand& b) const {
        if (c.bin >= 0 && bin[c.bin].child[0] >= 0) {
            a = of_bin(bin[c.bin].child[0]);
            b = of_bin(bin[c.bin].child[1]);
        } else {
            uint32_t h = c.count / 2;
            a = of_range(c.first, h);
            b = of_range(c.first + h, c.count - h);
        }
    }

    // The slot candidates of c's wide node: c's two halves (or c itself when it is a
    // leaf), then the expandable slot of largest surface area split again until W slots
    // are used.
    uint32_t slots(const Cand& c, Cand (&cands)[8]) const {
        uint32_t nc = 0;
        if (expandable(c)) {
            expand(c, cands[0], cands[1]);
            nc = 2;
        } else {
            cands[nc++] = c;
        }
        while (nc < W) {
            int best = -1;
            float best_area = -1.0f;
            for (uint32_t i = 0; i < nc; ++i) {
                if (!expandable(cands[i])) continue;
                float a = cands[i].box.area();
                if (!(a <= best_area)) {
                    best = static_cast<int>(i);
                    best_area = a;
                }
            }
            if (best < 0) break;
            Cand a, b;
            expand(cands[best], a, b);
            for (uint32_t i = nc; i > static_cast<uint32_t>(best) + 1; --i) cands[i] = cands[i - 1];
            cands[best] = a;
            cands[best + 1] = b;
            ++nc;
        }
        return nc;
    }

    // Wide nodes in the subtree of candidate c (c expandable, or the root).
    uint32_t count(const Cand& c) const {
        Cand cs[8];
        const uint32_t nc = slots(c, cs);
        uint32_t n = 1;
        for (uint32_t j = 0; j < nc; ++j)
            if (expandable(cs[j])) n += count(cs[j]);
        return n;
    }

    // Writes slot j of node idx: its box and reference (empty slots get an empty box).
    void put_slot(uint32_t idx, uint32_t j, const Box& bx, int32_t ref) {
        float* node = &out[static_cast<size_t>(idx) * 8 * W];
        for (int a = 0; a < 3; ++a) {
            node[a * W + j] = bx.lo[a];
            node[(3 + a) * W + j] = bx.hi[a];
        }
        std::memcpy(&node[6 * W + j], &ref, 4);
    }
    static int32_t leaf_ref(const Cand& k) { return ~static_cast<int32_t>((k.first << LEAF_COUNT_BITS) | (k.count - 1)); }

    // Writes c's wide node at `idx` and its subtree depth first from `next` (the order a
    // serial emission gives); returns the subtree's worst-case stack use.
    uint32_t emit_at(const Cand& c, uint32_t idx, uint32_t& next) {
        Cand cs[8];
        const uint32_t nc = slots(c, cs);
        uint32_t sub_max = 0;
        for (uint32_t j = 0; j < W; ++j) {
            if (j >= nc) {
                put_slot(idx, j, Box::empty(), ~0);  // unused: its box is empty
            } else if (!expandable(cs[j])) {
                put_slot(idx, j, cs[j].box, leaf_ref(cs[j]));
            } else {
                const uint32_t ci = next++;
                sub_max = std::max(sub_max, emit_at(cs[j], ci, next));
                put_slot(idx, j, cs[j].box, static_cast<int32_t>(ci));
            }
        }
        return nc - 1 + sub_max;
    }

    // The whole tree from `root`; returns its worst-case stack use.  For large trees the
    // top two levels are expanded first, the subtrees below them counted and written on
    // the pass pool at the indices a serial emission would give them.
    uint32_t build(const Cand& root, unsigned threads) {
        if (threads <= 1 || root.count < RefBuilder::SPLIT_PASS) {
            out.assign(static_cast<size_t>(count(root)) * 8 * W, 0.0f);
            uint32_t next = 1;
            return emit_at(root, 0, next);
        }
        struct Top {
            Cand cs[8];
            uint32_t nc = 0;
            int32_t kid[8];  // >= 0: a top node; -1: a leaf; <= -2: frontier subtree -(kid + 2)
        };
        std::vector<Top> top;
        std::vector<Cand> frontier;
        std::function<uint32_t(const Cand&, int)> plan = [&](const Cand& c, int depth) -> uint32_t {
            const uint32_t t = static_cast<uint32_t>(top.size());
            top.emplace_back();
            Top node;
            node.nc = slots(c, node.cs);
            for (uint32_t j = 0; j < node.nc; ++j) {
                if (!expandable(node.cs[j])) {
                    node.kid[j] = -1;
                } else if (depth + 1 < 2) {
                    node.kid[j] = static_cast<int32_t>(plan(node.cs[j], depth + 1));
                } else {
                    node.kid[j] = -2 - static_cast<int32_t>(frontier.size());
                    frontier.push_back(node.cs[j]);
                }
            }
            top[t] = node;
            return t;
        };
        plan(root, 0);
        const size_t nf = frontier.size();
        std::vector<uint32_t> fcount(nf), fbase(nf), fsu(nf, 0), tidx(top.size());
        RefBuilder::in_parts(nf, static_cast<unsigned>(nf), [&](unsigned, size_t b, size_t e) {
            for (size_t f = b; f < e; ++f) fcount[f] = count(frontier[f]);
        });
        uint32_t next = 0;  // depth-first indices, as a serial emission assigns them
        std::function<void(uint32_t)> number = [&](uint32_t t) {
            tidx[t] = next++;
            for (uint32_t j = 0; j < top[t].nc; ++j) {
                const int32_t k = top[t].kid[j];
                if (k >= 0) {
                    number(static_cast<uint32_t>(k));
                } else if (k <= -2) {
                    fbase[-2 - k] = next;
                    next += fcount[-2 - k];
                }
            }
        };
        number(0);
        out.assign(static_cast<size_t>(next) * 8 * W, 0.0f);
        RefBuilder::in_parts(nf, static_cast<unsigned>(nf), [&](unsigned, size_t b, size_t e) {
            for (size_t f = b; f < e; ++f) {
                uint32_t nx = fbase[f] + 1;
                fsu[f] = emit_at(frontier[f], fbase[f], nx);
            }
        });
        std::function<uint32_t(uint32_t)> write = [&](uint32_t t) -> uint32_t {
            const Top& node = top[t];
            uint32_t sub_max = 0;
            for (uint32_t j = 0; j < W; ++j) {
                if (j >= node.nc) {
                    put_slot(tidx[t], j, Box::empty(), ~0);
                } else if (node.kid[j] == -1) {
                    put_slot(tidx[t], j, node.cs[j].box, leaf_ref(node.cs[j]));
                } else if (node.kid[j] >= 0) {
                    sub_max = std::max(sub_max, write(static_cast<uint32_t>(node.kid[j])));
                    put_slot(tidx[t], j, node.cs[j].box, static_cast<int32_t>(tidx[node.kid[j]]));
                } else {
                    const size_t f = static_cast<size_t>(-2 - node.kid[j]);
                    sub_max = std::max(sub_max, fsu[f]);
                    put_slot(tidx[t], j, node.cs[j].box, static_cast<int32_t>(fbase[f]));
                }
            }
            return node.nc - 1 + sub_max;
        };
        return write(0);
    }
};

}  // namespace

static bool build_lobes(const gr_material_desc& d, DevMaterial& m, std::string& err) {
    std::memset(&m, 0, sizeof(m));
    auto set3 = [](float* dst, V3 v) {
        dst[0] = v.x;
        dst[1] = v.y;
        dst[2] = v.z;
    };
    switch (d.kind) {
        case GR_MATERIAL_DIFFUSE_LIGHT:
            m.has_light = 1;
            set3(m.emission, V3{d.incandescence[0], d.incandescence[1], d.incandescence[2]});
            set3(m.display, V3{d.incandescence[0], d.incandescence[1], d.incandescence[2]});
            return true;
        case GR_MATERIAL_DIFFUSE:
            set3(m.display, v3one());
            m.n_lobes = 1;
            m.lobe[0].type = L_PERFECT_DIFFUSE;
            m.lobe[0].kind = LOBE_DIFFUSE | LOBE_REFLECTION;
            return true;
        case GR_MATERIAL_MIRROR:
            set3(m.display, v3one());
            m.n_lobes = 1;
            m.lobe[0].type = L_PERFECT_MIRROR;
            m.lobe[0].kind = LOBE_SPECULAR | LOBE_REFLECTION;
            return true;
        case GR_MATERIAL_DISNEY:
            break;
        default:
            err = "unknown material kind " + std::to_string(d.kind);
            return false;
    }
    // DisneyMaterialBuilder::build (material/material.rs:292-333)
    V3 base = V3{d.base_color[0], d.base_color[1], d.base_color[2]};
    float dw = (1.0f - d.metallic) * (1.0f - d.specular_trans);
    float tw = (1.0f - d.metallic) * d.specular_trans;
    // GgxDistribution::new (material/util.rs:128-133)
    float aspect = sqrtf(1.0f - d.anisotropic * 0.9f);
    float ax = fmaxf(0.001f, d.roughness * d.roughness / aspect);
    float ay = fmaxf(0.001f, d.roughness * d.roughness * aspect);
    float ior_adj = fmaxf(d.ior, 1.01f);
    int n = 0;
    if (dw > 0.0f) {  // DisneyDiffuseRefl::new (lobes.rs:83-90)
        DevLobe& L = m.lobe[n++];
        L.type = L_DISNEY_DIFFUSE;
        L.kind = LOBE_DIFFUSE | LOBE_REFLECTION;
        set3(L.c0, base * dw);
        set3(L.c1, (d.sheen * dw) * vlerp(v3one(), tint(base), d.sheen_tint));
        L.p[0] = d.roughness;
    }
    if (d.ior > 1.0f) {  // DisneySpecularRefl::new_aniso (lobes.rs:212-226), DisneyFresnel::new (util.rs:64-69)
        DevLobe& L = m.lobe[n++];
        L.type = L_GGX_DISNEY;
        L.kind = LOBE_GLOSSY | LOBE_REFLECTION;
        set3(L.c0, base);
        set3(L.c1, vlerp(v3one(), tint(base), d.specular_tint));
        L.p[0] = ax;
        L.p[1] = ay;
        L.p[2] = ior_adj;
        L.p[3] = d.metallic;
    }
    if (d.clearcoat > 0.0f) {  // DisneyClearcoatRefl::new (lobes.rs:232-242), Gtr1Distribution::new
        DevLobe& L = m.lobe[n++];
        L.type = L_GTR1_SCHLICK;
        L.kind = LOBE_GLOSSY | LOBE_REFLECTION;
        set3(L.c0, (0.25f * d.clearcoat) * v3one());
        set3(L.c1, 0.04f * v3one());
        L.p[0] = lerp(0.1f, 0.001f, d.clearcoat_gloss);
    }
    if (tw > 0.0f) {  // DisneySpecularTrans::new_aniso (lobes.rs:258-268)
        DevLobe& L = m.lobe[n++];
        L.type = L_SPECULAR_TRANS;
        L.kind = LOBE_GLOSSY | LOBE_TRANSMISSION;
        set3(L.c0, tw * vsqrt(base));
        L.p[0] = ax;
        L.p[1] = ay;
        L.p[2] = ior_adj;
    }
    m.n_lobes = n;
    set3(m.display, base);
    return true;
}

bool build_material(const gr_material_desc& d, DevMaterial& m, std::string& err) {
    if (!build_lobes(d, m, err)) return false;
    // The shading sort's key for the material's mixture: its lobe count and types.
    m.lobe_set = static_cast<uint32_t>(m.n_lobes);
    for (int j = 0; j < m.n_lobes; ++j) m.lobe_set = m.lobe_set * 8u + static_cast<uint32_t>(m.lobe[j].type);
    return true;
}

static void put_bits(float* dst, uint32_t v) { std::memcpy(dst, &v, 4); }

// FNV-1a over the binary tree in depth-first order, left child first: each node's box,
// then a leaf's component count and (prim, component) ids, or an inner node's tag.
static uint64_t tree_hash(const BinNodes& nodes, int32_t root, const std::vector<Rec, NoInitAlloc<Rec>>& recs,
                          const std::vector<Item>& items) {
    uint64_t h = 1469598103934665603ull;
    auto add = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    std::vector<int32_t> stack{root};
    while (!stack.empty()) {
        const BinNode& nd = nodes[stack.back()];
        stack.pop_back();
        add(nd.box.lo, sizeof(nd.box.lo));
        add(nd.box.hi, sizeof(nd.box.hi));
        if (nd.child[0] < 0) {
            const uint32_t tag = 1, count = nd.count;
            add(&tag, 4);
            add(&count, 4);
            for (uint32_t j = 0; j < nd.count; ++j) {
                const Item& it = items[recs[nd.first + j].id & ID_MASK];
                const uint32_t pc[2] = {it.prim, it.comp};
                add(pc, sizeof(pc));
            }
        } else {
            const uint32_t tag = 0;
            add(&tag, 4);
            stack.push_back(nd.child[1]);
            stack.push_back(nd.child[0]);
        }
    }
    return h;
}

bool build_scene(const gr_scene_desc& desc, HostBuild& out, std::string& err, bool want_tree_hash) {
    out = HostBuild();
    uint32_t W = desc.bvh_width ? desc.bvh_width : 4;
    if (W != 2 && W != 4 && W != 8) {
        err = "bvh_width must be 2, 4 or 8";
        return false;
    }
    uint32_t L = desc.leaf_size ? desc.leaf_size : 2;  // 2 measured fastest (width 4) on the bench workload
    if (L < 1 || L > static_cast<uint32_t>(MAX_LEAF_PRIMS)) {
        err = "leaf_size must be in [1, 16]";
        return false;
    }
    out.width = W;
    for (uint32_t i = 0; i < desc.num_materials; ++i) {
        DevMaterial m;
        if (!build_material(desc.materials[i], m, err)) return false;
        out.materials.push_back(m);
    }
    if (desc.num_prims && !desc.prims) {
        err = "null prims";
        return false;
    }
    // Component list in prim order (Bvh::build, bvh.rs:340-350), with mesh data offsets.
    std::vector<Item> items;
    {
        size_t total = 0;
        for (uint32_t p = 0; p < desc.num_prims && desc.prims; ++p)
            total += desc.prims[p].kind == GR_PRIM_MESH ? desc.prims[p].num_tris : 1;
        items.reserve(total);
    }
    std::vector<uint32_t> vbase(desc.num_prims, 0), nbase(desc.num_prims, 0), ubase(desc.num_prims, 0);
    uint32_t nrm_total = 0, uv_total = 0;
    for (uint32_t p = 0; p < desc.num_prims; ++p) {
        const gr_prim_desc& d = desc.prims[p];
        if (d.material >= desc.num_materials) {
            err = "prim " + std::to_string(p) + ": material index out of range";
            return false;
        }
        out.prim_material.push_back(d.material);
        if (d.kind == GR_PRIM_SPHERE) {
            if (!(d.radius > 0.0f)) {
                err = "sphere radius must be > 0";
                return false;
            }
            Item it;
            it.prim = p;
            it.comp = 0;
            for (int k = 0; k < 3; ++k) {  // Sphere::bbox_world (sphere.rs:47-58)
                it.box.lo[k] = d.center[k] - d.radius;
                it.box.hi[k] = d.center[k] + d.radius;
                it.cen[k] = 0.5f * it.box.lo[k] + 0.5f * it.box.hi[k];  // bvh.rs:26
            }
            items.push_back(it);
        } else if (d.kind == GR_PRIM_MESH) {
            if (d.num_tris == 0 || !d.vertices || !d.tri_vertices) {
                err = "mesh " + std::to_string(p) + " has no triangles";
                return false;
            }
            // Triangle t: its index checks (0: fine, else the first that fails) and its
            // item.  Large meshes run on threads; the error reported is the first
            // failing triangle's, as in a serial pass.
            const size_t ibase = items.size();
            items.resize(ibase + d.num_tris);
            auto triangle = [&](uint32_t t) -> int {
                for (int k = 0; k < 3; ++k)
                    if (d.tri_vertices[3 * t + k] >= d.num_vertices) return 1;
                if (d.tri_normals && d.tri_normals[3 * t] != GR_NO_INDEX)
                    for (int k = 0; k < 3; ++k)
                        if (d.tri_normals[3 * t + k] >= d.num_normals) return 2;
                if (d.tri_uvs)
                    for (int k = 0; k < 3; ++k)
                        if (d.tri_uvs[3 * t + k] >= d.num_uvs) return 3;
                Item& it = items[ibase + t];
                it.prim = p;
                it.comp = t;
                it.box = Box::empty();  // Mesh::bbox_world (mesh.rs:262-268)
                for (int k = 0; k < 3; ++k) it.box.grow(d.vertices + 3 * d.tri_vertices[3 * t + k]);
                for (int k = 0; k < 3; ++k) it.cen[k] = 0.5f * it.box.lo[k] + 0.5f * it.box.hi[k];  // bvh.rs:26
                return 0;
            };
            uint64_t bad = UINT64_MAX;  // (triangle << 2) | check of the first failure
            const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
            if (d.num_tris >= RefBuilder::SPLIT_PASS && hw > 1) {
                std::vector<uint64_t> part_bad(hw, UINT64_MAX);
                RefBuilder::in_parts(d.num_tris, hw, [&](unsigned k, size_t b, size_t e) {
                    for (size_t t = b; t < e; ++t)
                        if (int c = triangle(static_cast<uint32_t>(t))) {
                            part_bad[k] = (static_cast<uint64_t>(t) << 2) | static_cast<uint64_t>(c);
                            break;
                        }
                });
                for (uint64_t v : part_bad) bad = std::min(bad, v);
            } else {
                for (uint32_t t = 0; t < d.num_tris && bad == UINT64_MAX; ++t)
                    if (int c = triangle(t)) bad = (static_cast<uint64_t>(t) << 2) | static_cast<uint64_t>(c);
            }
            if (bad != UINT64_MAX) {
                const int c = static_cast<int>(bad & 3u);
                err = c == 1 ? "vertex index out of range" : (c == 2 ? "normal index out of range" : "uv index out of range");
                return false;
            }
            if (d.tri_normals && d.num_normals) {
                out.any_normals = true;
                nbase[p] = nrm_total;
                nrm_total += d.num_normals;
                out.normals.insert(out.normals.end(), d.normals, d.normals + 3 * d.num_normals);
            }
            if (d.tri_uvs && d.num_uvs) {
                out.any_uvs = true;
                ubase[p] = uv_total;
                uv_total += d.num_uvs;
                out.uvs.insert(out.uvs.end(), d.uvs, d.uvs + 2 * d.num_uvs);
            }
        } else {
            err = "unknown prim kind";
            return false;
        }
    }
    out.num_components = items.size();
    if (items.empty()) {
        err = "scene has no components";
        return false;
    }
    if (items.size() >= (1u << (31 - LEAF_COUNT_BITS))) {
        err = "too many components";
        return false;
    }

    if (desc.build != GR_BUILD_HOST_SAH && desc.build != GR_BUILD_DEVICE_LBVH) {
        err = "build must be GR_BUILD_HOST_SAH or GR_BUILD_DEVICE_LBVH";
        return false;
    }
    out.device_build = desc.build == GR_BUILD_DEVICE_LBVH;

    // Primitive records: in leaf order for the host build, in component order for the
    // device build (which sorts them itself, bvh_build.cu).
    out.prims.resize(items.size() * 12);  // not filled: put_record writes all 12 floats
    if (out.any_normals) out.tri_normal_idx.assign(items.size() * 3, NO_INDEX);
    if (out.any_uvs) out.tri_uv_idx.assign(items.size() * 3, NO_INDEX);
    auto put_record = [&](size_t k, const Item& it) {
        const gr_prim_desc& d = desc.prims[it.prim];
        float* r = &out.prims[k * 12];
        if (d.kind == GR_PRIM_SPHERE) {
            r[0] = d.center[0];
            r[1] = d.center[1];
            r[2] = d.center[2];
            put_bits(r + 3, it.prim);
            r[4] = d.radius;
            r[5] = r[6] = 0.0f;
            put_bits(r + 7, 0);
            r[8] = r[9] = r[10] = 0.0f;
            put_bits(r + 11, PRIM_SPHERE);
        } else {
            const float* a = d.vertices + 3 * d.tri_vertices[3 * it.comp];
            const float* b = d.vertices + 3 * d.tri_vertices[3 * it.comp + 1];
            const float* c = d.vertices + 3 * d.tri_vertices[3 * it.comp + 2];
            for (int q = 0; q < 3; ++q) {
                r[q] = c[q];
                r[4 + q] = a[q] - c[q];  // edge1 = a - c (mesh.rs:278)
                r[8 + q] = b[q] - c[q];  // edge2 = b - c
            }
            put_bits(r + 3, it.prim);
            put_bits(r + 7, it.comp);
            put_bits(r + 11, PRIM_TRIANGLE);
            if (out.any_normals && d.tri_normals && d.tri_normals[3 * it.comp] != GR_NO_INDEX)
                for (int q = 0; q < 3; ++q) out.tri_normal_idx[3 * k + q] = nbase[it.prim] + d.tri_normals[3 * it.comp + q];
            if (out.any_uvs && d.tri_uvs)
                for (int q = 0; q < 3; ++q) out.tri_uv_idx[3 * k + q] = ubase[it.prim] + d.tri_uvs[3 * it.comp + q];
        }
    };

    if (out.device_build) {
        out.leaf_size = L;
        out.item_boxes.resize(items.size() * 6);
        auto records = [&](unsigned, size_t b, size_t e) {
            for (size_t k = b; k < e; ++k) {
                put_record(k, items[k]);
                for (int a = 0; a < 3; ++a) {
                    out.item_boxes[6 * k + a] = items[k].box.lo[a];
                    out.item_boxes[6 * k + 3 + a] = items[k].box.hi[a];
                }
            }
        };
        const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        if (items.size() >= RefBuilder::SPLIT_PASS && hw > 1)
            RefBuilder::in_parts(items.size(), hw, records);
        else
            records(0, 0, items.size());
    } else {
        std::vector<Rec, NoInitAlloc<Rec>> recs(items.size());  // every element written below
        auto fill = [&](unsigned, size_t b, size_t e) {
            for (size_t k = b; k < e; ++k) {
                recs[k].box = items[k].box;
                std::memcpy(recs[k].cen, items[k].cen, sizeof(recs[k].cen));
                recs[k].id = static_cast<uint32_t>(k);
            }
        };
        RefBuilder rb(recs.data(), recs.size());
        if (recs.size() >= RefBuilder::SPLIT_PASS && rb.threads > 1)
            RefBuilder::in_parts(recs.size(), rb.threads, fill);
        else
            fill(0, 0, recs.size());
        int32_t root = rb.build(recs.data(), recs.size());
        out.num_binary_nodes = rb.node_count();
        if (want_tree_hash) out.tree_hash = tree_hash(rb.nodes, root, recs, items);
        std::vector<Box, NoInitAlloc<Box>> comp_box(items.size());  // written by the records pass
        auto records = [&](unsigned, size_t b, size_t e) {
            for (size_t k = b; k < e; ++k) {
                const Item& it = items[recs[k].id & ID_MASK];
                comp_box[k] = it.box;
                put_record(k, it);
            }
        };
        if (recs.size() >= RefBuilder::SPLIT_PASS && rb.threads > 1)
            RefBuilder::in_parts(recs.size(), rb.threads, records);
        else
            records(0, 0, recs.size());
        Collapser col(rb.nodes, comp_box, W, L, out.nodes);
        out.stack_depth = col.build(col.of_bin(root), rb.threads) + 1;
        if (out.stack_depth > static_cast<uint32_t>(MAX_STACK)) {
            err = "BVH too deep: traversal needs " + std::to_string(out.stack_depth) + " stack entries (limit " +
                  std::to_string(MAX_STACK) + ")";
            return false;
        }
        out.num_wide_nodes = out.nodes.size() / (8 * W);
    }

    // Light tables (Bvh::build caches light prims, bvh.rs:364-370; Mesh area CDF, mesh.rs:161-170).
    for (uint32_t p = 0; p < desc.num_prims; ++p) {
        if (!out.materials[desc.prims[p].material].has_light) continue;
        const gr_prim_desc& d = desc.prims[p];
        LightRec lr;
        std::memset(&lr, 0, sizeof(lr));
        lr.prim = p;
        if (d.kind == GR_PRIM_SPHERE) {
            lr.type = PRIM_SPHERE;
            lr.center[0] = d.center[0];
            lr.center[1] = d.center[1];
            lr.center[2] = d.center[2];
            lr.radius = d.radius;
        } else {
            lr.type = PRIM_TRIANGLE;
            lr.first_tri = static_cast<uint32_t>(out.light_cdf.size());
            lr.num_tris = d.num_tris;
            float total = 0.0f;
            size_t c0 = out.light_cdf.size();
            for (uint32_t t = 0; t < d.num_tris; ++t) {
                const float* a = d.vertices + 3 * d.tri_vertices[3 * t];
                const float* b = d.vertices + 3 * d.tri_vertices[3 * t + 1];
                const float* c = d.vertices + 3 * d.tri_vertices[3 * t + 2];
                V3 e1 = V3{a[0] - c[0], a[1] - c[1], a[2] - c[2]};
                V3 e2 = V3{b[0] - c[0], b[1] - c[1], b[2] - c[2]};
                total += 0.5f * magnitude(cross(e1, e2));  // Tri::area (mesh.rs:37-47)
                out.light_cdf.push_back(total);
                for (const float* v : {a, b, c}) {
                    out.light_tris.push_back(v[0]);
                    out.light_tris.push_back(v[1]);
                    out.light_tris.push_back(v[2]);
                    out.light_tris.push_back(0.0f);
                }
                for (int q = 0; q < 3; ++q) {
                    bool hn = d.tri_normals && d.tri_normals[3 * t] != GR_NO_INDEX;
                    out.light_tri_normal_idx.push_back(hn ? nbase[p] + d.tri_normals[3 * t + q] : NO_INDEX);
                    out.light_tri_uv_idx.push_back(d.tri_uvs ? ubase[p] + d.tri_uvs[3 * t + q] : NO_INDEX);
                }
            }
            for (size_t i = c0; i < out.light_cdf.size(); ++i) out.light_cdf[i] = out.light_cdf[i] / total;
            lr.area = total;
        }
        out.lights.push_back(lr);
    }
    return true;
}

}  // namespace gr
