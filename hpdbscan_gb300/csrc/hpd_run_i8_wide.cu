// Pipeline instantiation for int8_t points on grids of more than five dimensions
// (compiled apart from hpd_run_i8.cu to keep each translation unit short).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline_dims<int8_t, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
