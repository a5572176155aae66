// TEST INFRASTRUCTURE ONLY: a minimal stand-in for the spdlog logging library, which ReaDDy's headers
// include (include/readdy/common/logging.h) and which is not installed in this image.  It offers only
// the names ReaDDy uses -- a named logger with a level, and trace/debug/info/warn/error/critical calls
// that format with {fmt} -- so that ReaDDy's own sources compile unchanged against it (the plugin
// syntax check of the tests and the reference CPU kernel built as the timed baseline).  Messages at or
// above the logger's level go to stderr.
#pragma once
#include <fmt/format.h>

#include <cassert>  // spdlog's headers bring it in; ReaDDy's sources rely on that
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>  // spdlog's own headers bring it in; ReaDDy's common.h relies on that

namespace spdlog {
namespace level {
enum level_enum : int { trace = 0, debug = 1, info = 2, warn = 3, err = 4, critical = 5, off = 6 };
}
template <typename... Args>
using format_string_t = fmt::format_string<Args...>;

namespace sinks {
class sink {
public:
    virtual ~sink() = default;
};
}  // namespace sinks

class logger {
public:
    explicit logger(std::string name) : _name(std::move(name)) {}
    logger(std::string name, std::shared_ptr<sinks::sink>) : _name(std::move(name)) {}
    void set_level(level::level_enum l) { _level = l; }
    void set_pattern(const std::string &) {}
    level::level_enum level() const { return _level; }
    const std::string &name() const { return _name; }
    template <typename... A> void trace(format_string_t<A...> f, A &&...a) { log(level::trace, f, std::forward<A>(a)...); }
    template <typename... A> void debug(format_string_t<A...> f, A &&...a) { log(level::debug, f, std::forward<A>(a)...); }
    template <typename... A> void info(format_string_t<A...> f, A &&...a) { log(level::info, f, std::forward<A>(a)...); }
    template <typename... A> void warn(format_string_t<A...> f, A &&...a) { log(level::warn, f, std::forward<A>(a)...); }
    template <typename... A> void error(format_string_t<A...> f, A &&...a) { log(level::err, f, std::forward<A>(a)...); }
    template <typename... A> void critical(format_string_t<A...> f, A &&...a) { log(level::critical, f, std::forward<A>(a)...); }

private:
    template <typename... A>
    void log(level::level_enum l, format_string_t<A...> f, A &&...a) {
        if (l < _level) return;
        const std::string m = fmt::format(f, std::forward<A>(a)...);
        std::fprintf(stderr, "[%s] %s\n", _name.c_str(), m.c_str());
    }
    std::string _name;
    level::level_enum _level = level::warn;
};

namespace detail {
inline std::map<std::string, std::shared_ptr<logger>> &registry() {
    static std::map<std::string, std::shared_ptr<logger>> r;
    return r;
}
inline std::mutex &registry_mutex() {
    static std::mutex m;
    return m;
}
}  // namespace detail

inline std::shared_ptr<logger> get(const std::string &name) {
    std::lock_guard<std::mutex> g(detail::registry_mutex());
    auto it = detail::registry().find(name);
    return it == detail::registry().end() ? nullptr : it->second;
}
inline void register_logger(std::shared_ptr<logger> l) {
    std::lock_guard<std::mutex> g(detail::registry_mutex());
    detail::registry()[l->name()] = l;
}
inline void drop(const std::string &name) {
    std::lock_guard<std::mutex> g(detail::registry_mutex());
    detail::registry().erase(name);
}
inline std::shared_ptr<logger> stdout_color_mt(const std::string &name) {
    auto l = std::make_shared<logger>(name);
    register_logger(l);
    return l;
}
inline std::shared_ptr<logger> stderr_color_mt(const std::string &name) { return stdout_color_mt(name); }
inline void set_level(level::level_enum) {}
}  // namespace spdlog
