// Pipeline instantiation for uint16_t points (upstream cluster<uint16_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<uint16_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
