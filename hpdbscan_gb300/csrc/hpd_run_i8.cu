// Pipeline instantiation for int8_t points (upstream cluster<int8_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<int8_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
