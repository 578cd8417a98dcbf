// Pipeline instantiation for float points on grids of more than five dimensions
// (compiled apart from hpd_run_f32.cu to keep each translation unit short).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline_dims<float, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
