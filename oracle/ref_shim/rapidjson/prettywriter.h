// Stand-in for rapidjson's pretty writer (writes nothing).
#pragma once
#include "document.h"
namespace rapidjson {
template <typename OS>
struct PrettyWriter {
    explicit PrettyWriter(OS&) {}
};
template <typename OS>
struct Writer {
    explicit Writer(OS&) {}
};
}  // namespace rapidjson
