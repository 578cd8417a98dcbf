// Pipeline instantiation for int32_t points (upstream cluster<int32_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<int32_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
