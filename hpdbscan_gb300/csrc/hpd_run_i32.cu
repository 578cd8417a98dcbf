// Pipeline instantiation for int32_t points (upstream cluster<int32_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_i32_wide.cu
extern template int run_pipeline_dims<int32_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<int32_t, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<int32_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
