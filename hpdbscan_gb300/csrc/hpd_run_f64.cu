// Pipeline instantiation for double points (upstream cluster<double>; the Python
// binding's path, swig/hpdbscan.i:27).
#include "hpd_pipeline.cuh"

namespace hpd {
// grids past five dimensions: hpd_run_f64_wide.cu
extern template int run_pipeline_dims<double, true>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline_dims<double, false>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
template int run_pipeline<double>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
