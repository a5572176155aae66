// TEST INFRASTRUCTURE ONLY: spdlog's bridge to {fmt}'s ostream support (see spdlog/spdlog.h here).
#pragma once
#include <fmt/ostream.h>
