// Pipeline instantiation for int16_t points (upstream cluster<int16_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_i16_wide.cu
extern template int run_pipeline_dims<int16_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<int16_t, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<int16_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
