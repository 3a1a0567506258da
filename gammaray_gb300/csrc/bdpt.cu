// Wavefront BDPT (render/integrators.rs:102-418).
#include "runtime.hpp"

namespace gr {

gr_status render_bdpt(gr_scene*, const RenderJob&, cudaStream_t) {
    set_error("BDPT is not built yet");
    return GR_ERR_UNSUPPORTED;
}

}  // namespace gr
