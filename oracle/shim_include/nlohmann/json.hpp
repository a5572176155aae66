// TEST INFRASTRUCTURE ONLY: stand-in for the nlohmann JSON library, which ReaDDy's kernel configuration
// header names (include/readdy/api/KernelConfiguration.h) and which is not installed in this image.  Only
// the type is declared: ReaDDy's headers use it in declarations, and the sources compiled against it here
// take their configuration from defaults instead of a JSON string.
#pragma once
namespace nlohmann {
class json;
}
