// Pipeline instantiation for double points (upstream cluster<double>; the Python
// binding's path, swig/hpdbscan.i:27).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<double>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
