// Pipeline instantiation for float points (upstream cluster<float>).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_f32_wide.cu
extern template int run_pipeline_dims<float, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<float, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<float>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
