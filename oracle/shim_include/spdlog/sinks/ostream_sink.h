// TEST INFRASTRUCTURE ONLY: stand-in for spdlog's ostream sink (see spdlog/spdlog.h here).
#pragma once
#include <ostream>

#include "../spdlog.h"

namespace spdlog::sinks {
template <typename Mutex>
class ostream_sink : public sink {
public:
    explicit ostream_sink(std::ostream &, bool = false) {}
};
using ostream_sink_mt = ostream_sink<std::mutex>;
using ostream_sink_st = ostream_sink<void>;
}  // namespace spdlog::sinks
