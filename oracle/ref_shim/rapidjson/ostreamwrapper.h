// Stand-in for rapidjson's ostream wrapper.
#pragma once
#include <ostream>
#include "document.h"
namespace rapidjson {
struct OStreamWrapper {
    explicit OStreamWrapper(std::ostream&) {}
};
}  // namespace rapidjson
