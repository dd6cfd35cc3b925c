// Stand-in for rapidjson's string buffer.
#pragma once
#include "document.h"
namespace rapidjson {
struct StringBuffer {
    const char* GetString() const { return ""; }
};
}  // namespace rapidjson
