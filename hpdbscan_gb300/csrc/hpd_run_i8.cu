// Pipeline instantiation for int8_t points (upstream cluster<int8_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_i8_wide.cu
extern template int run_pipeline_dims<int8_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<int8_t, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<int8_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
