// Pipeline instantiation for int64_t points (upstream cluster<int64_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_i64_wide.cu
extern template int run_pipeline_dims<int64_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<int64_t, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<int64_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
