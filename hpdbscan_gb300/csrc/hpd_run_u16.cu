// Pipeline instantiation for uint16_t points (upstream cluster<uint16_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_u16_wide.cu
extern template int run_pipeline_dims<uint16_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<uint16_t, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<uint16_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
