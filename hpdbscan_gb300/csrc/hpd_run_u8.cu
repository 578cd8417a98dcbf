// Pipeline instantiation for uint8_t points (upstream cluster<uint8_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<uint8_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
