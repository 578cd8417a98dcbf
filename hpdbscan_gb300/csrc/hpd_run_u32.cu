// Pipeline instantiation for uint32_t points (upstream cluster<uint32_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<uint32_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
