// Stand-in for spdlog's console sink.
#pragma once
#include "../spdlog.h"
namespace spdlog {
namespace sinks {
struct stdout_color_sink_mt : sink {
};
}  // namespace sinks
}  // namespace spdlog
