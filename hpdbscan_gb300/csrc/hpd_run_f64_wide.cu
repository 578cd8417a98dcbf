// Pipeline instantiation for double points on grids of more than five dimensions
// (compiled apart from hpd_run_f64.cu to keep each translation unit short).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline_dims<double, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
