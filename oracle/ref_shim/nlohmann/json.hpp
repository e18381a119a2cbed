// Stand-in (test infrastructure for oracle/_ref).
#pragma once
#include <nlohmann/json_fwd.hpp>
