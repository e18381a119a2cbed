// Stand-in glm header (test infrastructure for oracle/_ref); everything lives in detail_vec.hpp.
#pragma once
#include <glm/detail_vec.hpp>
