// Batched rendering and the serving loop.
#include "runtime.hpp"

using namespace gr;

extern "C" {

gr_status gr_render_batch(const gr_job* jobs, uint32_t n, const gr_batch_options*) {
    if (n && !jobs) {
        set_error("null jobs");
        return GR_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t i = 0; i < n; ++i) {
        gr_status s = gr_render(jobs[i].scene, &jobs[i].camera, &jobs[i].params, jobs[i].film);
        if (s != GR_OK) return s;
    }
    return GR_OK;
}

static gr_status unsupported() {
    set_error("serving is not built yet");
    return GR_ERR_UNSUPPORTED;
}
gr_status gr_server_create(const gr_server_options*, gr_server**) { return unsupported(); }
gr_status gr_server_destroy(gr_server*) { return unsupported(); }
gr_status gr_server_submit(gr_server*, const gr_request*, uint64_t*) { return unsupported(); }
gr_status gr_server_step(gr_server*, double) { return unsupported(); }
gr_status gr_server_poll(gr_server*, uint64_t, gr_request_status*) { return unsupported(); }
gr_status gr_server_cancel(gr_server*, uint64_t) { return unsupported(); }
gr_status gr_server_take(gr_server*, uint64_t, float*, float*) { return unsupported(); }

}  // extern "C"
