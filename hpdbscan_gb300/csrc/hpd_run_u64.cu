// Pipeline instantiation for uint64_t points (upstream cluster<uint64_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_u64_wide.cu
extern template int run_pipeline_dims<uint64_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<uint64_t, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<uint64_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
