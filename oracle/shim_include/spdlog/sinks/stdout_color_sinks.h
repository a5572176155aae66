// TEST INFRASTRUCTURE ONLY: stand-in for spdlog's colour console sinks (see spdlog/spdlog.h here).
#pragma once
#include "../spdlog.h"
