// Stand-in (test infrastructure for oracle/_ref): nothing beyond fmt/format.h is needed.
#pragma once
#include <fmt/format.h>
