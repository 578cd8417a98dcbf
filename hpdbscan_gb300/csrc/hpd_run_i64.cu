// Pipeline instantiation for int64_t points (upstream cluster<int64_t>, src/hpdbscan.cpp:19-30).
#include "hpd_pipeline.cuh"

namespace hpd {
template int run_pipeline<int64_t>(const Request&, Arena&, Arena&, Timers*, RunInfo&, std::string&);
}
