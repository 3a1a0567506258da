// Multi-job wavefront engine: the machinery behind gr_render_batch and gr_server_*.
//
// Many renders ("jobs": a scene, a camera, settings and a film) share one wavefront.
// Each job's work is a list of units, one per pass; units are issued in a global order
// (round-robin over jobs, pass by pass).  A live path's state travels with its ray in
// the queue; global path p has slot p mod ring of a ring holding its film position and,
// once it finishes, its radiance.  Every iteration:
//   plan    (1 thread) picks the finished units to gather (consecutive from the oldest)
//           and how many new paths to issue (queue room, ring slots already gathered)
//   gather  splats the picked units into their films from their ring slots (the
//           deterministic tile gather); each film tile adds its job's units in pass
//           order, every resident block taking (tile, units) items from a counter
//   fill    starts the next paths in their slots (jitter, camera ray) and queues them
//   extend  closest hit for the queued rays of all jobs
//   shade   path-tracer shading per job, material-sorted; finished paths leave their
//           radiance in their slot and count their unit done
// All launches have fixed grids and read their sizes from device memory, so an
// iteration pair is captured once in a CUDA graph and replayed until every unit is
// gathered.  A job's passes are gathered in pass order, so each film is identical to the
// film the job gets when it renders alone.
#pragma once

#include <cstdint>
#include <vector>

#include "runtime.hpp"

namespace gr {

struct alignas(16) DevJob {
    DeviceScene scene;
    DevCamera cam;
    float4* film;
    uint64_t seed;
    uint32_t width, height, npix;
    uint32_t display;  // display-colour integrator
    uint32_t max_depth, rr_depth, rr_aggr;
    uint32_t live;  // 0: cancelled, its paths are dropped
};

struct DevUnit {
    uint64_t prefix;  // global index of the unit's first path
    uint32_t job;
    uint32_t pass;
    uint32_t npix;
    uint32_t pad;
};

constexpr int GATHER_MAX = 256;

struct EngineCtl {
    unsigned long long paths_total;  // paths of all units appended so far
    unsigned long long gcur;         // next path to issue
    unsigned long long gather_lo_prefix;
    unsigned long long fill_base;
    unsigned long long rays;
    uint32_t units_count;
    uint32_t g_lo;  // oldest unit not yet gathered
    uint32_t q[2];
    uint32_t fill_n;
    uint32_t fill_qbase;  // queue position of the fill's first camera ray
    uint32_t fill_ulo, fill_uhi;  // units holding the paths of this fill: [fill_ulo, fill_uhi]
    uint32_t gather_n;       // units to gather this iteration, grouped by job
    uint32_t gather_groups;  // distinct jobs among them
    uint32_t done;
    int32_t err;
    uint32_t iter;
    uint32_t fetch;  // rays handed out by the refilling extension kernel this iteration
    uint32_t gather_next;  // film-tile items handed out by the gather this iteration
    // Set by the host (0 = none): gather as soon as every unit below this one has
    // finished, without waiting for a larger batch, so the request those units complete
    // is done within one iteration.
    uint32_t flush_unit;
    uint32_t gather_units[GATHER_MAX];      // unit indices, each job's units contiguous and in pass order
    uint32_t gather_group_first[GATHER_MAX];  // per group: first entry in gather_units
    uint32_t gather_group_count[GATHER_MAX];
    uint32_t gather_group_tiles[GATHER_MAX];  // per group: cumulative film tiles (exclusive prefix)
    uint32_t gather_tiles;                    // total film tiles of all groups
};

struct EngineConfig {
    uint32_t capacity = 1u << 21;  // path slots
    uint32_t width = 4;            // BVH width of every scene in the engine
    uint32_t block = 128;          // extension kernel block size (64, 128, 256)
    uint32_t ring = 0;             // path state slots (power of two); 0 = derived
};

class Engine {
  public:
    Engine() {}
    ~Engine();
    gr_status init(const EngineConfig& cfg, cudaStream_t st);
    // Appends a job and its units (one per pass).  Returns the job index.
    gr_status add_job(const DevJob& job, uint32_t first_pass, uint32_t passes, uint32_t& job_index);
    // Appends units of several jobs round-robin by pass: units[k] = (job, pass).
    gr_status append_units(const std::vector<std::pair<uint32_t, uint32_t>>& units);
    gr_status cancel_job(uint32_t job_index);
    // Sets EngineCtl::flush_unit (0 = none) for the iterations that follow.
    gr_status set_flush_unit(uint32_t unit);
    // Forgets every job and unit (buffers and the captured graph are kept).
    gr_status reset();
    // Runs iteration pairs (graph replays) until every appended unit is gathered,
    // `max_pairs` pairs ran, or the oldest ungathered unit reaches `stop_at_unit` (so a
    // caller waiting for the units before it hears of them within one pair).  Returns
    // whether all work is done.
    gr_status run(uint32_t max_pairs, bool& done, uint32_t stop_at_unit = 0xFFFFFFFFu);
    // Host copies of the control block and unit progress (synchronises the stream).
    gr_status read_ctl(EngineCtl& ctl);
    // The control block as the last run() left it (read there, no further sync), and the
    // graph pairs that run launched.
    const EngineCtl& last_ctl() const { return last_ctl_; }
    uint32_t last_pairs() const { return last_pairs_; }
    gr_status unit_done_counts(std::vector<uint32_t>& done);
    const std::vector<DevUnit>& units() const { return h_units_; }
    const std::vector<DevJob>& jobs() const { return h_jobs_; }
    uint32_t capacity() const { return cfg_.capacity; }
    uint32_t ring() const { return ring_; }  // path state slots; an image may use half
    const EngineConfig& config() const { return cfg_; }
    uint64_t rays() const { return last_rays_; }
    uint64_t device_bytes() const { return bytes_; }
    cudaStream_t stream() const { return st_; }

  private:
    gr_status record_pair();
    gr_status enqueue_iteration(int cur);
    EngineConfig cfg_;
    cudaStream_t st_ = nullptr;
    uint32_t ring_ = 0;
    DevBuf ctl_, jobs_, units_, unit_done_;
    DevBuf s_hot_, s_cold_;  // path state ring (see engine.cu)
    DevBuf q_slot_[2], q_o_[2], q_d_[2], q_state_[2], q_hit_;
    std::vector<DevJob> h_jobs_;
    std::vector<DevUnit> h_units_;
    uint32_t jobs_cap_ = 0, units_cap_ = 0;
    cudaGraphExec_t graph_ = nullptr;
    uint64_t last_rays_ = 0;
    EngineCtl last_ctl_{};
    uint32_t last_pairs_ = 0;
    uint64_t bytes_ = 0;
    uint64_t* h_pinned_ = nullptr;
};

// DeviceScene + camera + settings of a render as an engine job.
DevJob make_job(gr_scene* scene, const gr_camera& cam, const gr_render_params& p, uint32_t width, uint32_t height,
                float4* film);

}  // namespace gr
