// Stand-in for the part of spdlog's interface that Neon/core/tools/Logger.h uses:
// a named logger over a list of sinks, levels, and fmt-style "{}" messages.
// Messages at or above the logger's level (warn by default here) go to stderr.
#pragma once
#include <cstdio>
#include <iterator>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace spdlog {
namespace level {
enum level_enum { trace = 0, debug, info, warn, err, critical, off };
}
namespace sinks {
struct sink {
    virtual ~sink() = default;
    void set_pattern(const std::string&) {}
};
}  // namespace sinks
using sink_ptr = std::shared_ptr<sinks::sink>;

namespace detail {
inline void format_into(std::ostringstream& os, const char* f) { os << f; }
template <typename A, typename... R>
void format_into(std::ostringstream& os, const char* f, const A& a, const R&... r)
{
    for (; *f; ++f) {
        if (f[0] == '{' && f[1] == '}') {
            os << a;
            format_into(os, f + 2, r...);
            return;
        }
        os << *f;
    }
}
}  // namespace detail

class logger
{
   public:
    template <typename It>
    logger(std::string name, It, It) : mName(std::move(name))
    {
    }
    void set_level(level::level_enum l) { mLevel = l; }
    void flush_on(level::level_enum) {}
    template <typename... A>
    void log(level::level_enum l, const char* f, const A&... a)
    {
        if (l < mThreshold || l < mLevel) return;
        std::ostringstream os;
        detail::format_into(os, f, a...);
        std::fprintf(stderr, "[%s] %s\n", mName.c_str(), os.str().c_str());
    }
    template <typename S, typename... A>
    void trace(const S& f, const A&... a) { log(level::trace, as_c(f), a...); }
    template <typename S, typename... A>
    void debug(const S& f, const A&... a) { log(level::debug, as_c(f), a...); }
    template <typename S, typename... A>
    void info(const S& f, const A&... a) { log(level::info, as_c(f), a...); }
    template <typename S, typename... A>
    void warn(const S& f, const A&... a) { log(level::warn, as_c(f), a...); }
    template <typename S, typename... A>
    void error(const S& f, const A&... a) { log(level::err, as_c(f), a...); }
    template <typename S, typename... A>
    void critical(const S& f, const A&... a) { log(level::critical, as_c(f), a...); }

   private:
    static const char* as_c(const char* s) { return s; }
    static const char* as_c(const std::string& s) { return s.c_str(); }
    std::string        mName;
    level::level_enum  mLevel = level::trace;
    level::level_enum  mThreshold = level::warn;
};

inline void register_logger(std::shared_ptr<logger>) {}
}  // namespace spdlog
