// Pipeline instantiation for float points (upstream cluster<float>).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<float>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
