// Stand-in for spdlog's file sink (no file is written).
#pragma once
#include "../spdlog.h"
namespace spdlog {
namespace sinks {
struct basic_file_sink_mt : sink {
    basic_file_sink_mt(const std::string&, bool) {}
};
}  // namespace sinks
}  // namespace spdlog
