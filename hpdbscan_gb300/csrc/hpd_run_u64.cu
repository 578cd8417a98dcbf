// Pipeline instantiation for uint64_t points (upstream cluster<uint64_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<uint64_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
