// Pipeline instantiation for int16_t points (upstream cluster<int16_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<int16_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
